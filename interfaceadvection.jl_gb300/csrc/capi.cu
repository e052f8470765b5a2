// C-ABI of libintfadv_gb300 (declared in include/intfadv.h): handle life
// cycle, field binding, the VOF entry points and status read-back.
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstring>
#include <new>

#include "capi_internal.cuh"
#include "ff.cuh"

using namespace ia;

namespace {

__global__ void status_reset_k(DevStatus* s) {
    s->flags = 0;
    s->dir = 0;
    s->max_enc = 0ull;
    s->min_enc = ~0ull;
    s->max_key = 0ull;
    s->min_key = 0ull;
    for (int i = 0; i < 32; ++i) s->list_count[i] = 0;
}

}  // namespace

namespace ia {

static std::atomic<long long> g_launches{0};
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void note_launches(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long long launch_count() { return g_launches.load(std::memory_order_relaxed); }

int cuda_fail(cudaError_t e) {
    return e == cudaSuccess ? IA_OK : IA_ERR_CUDA;
}

int status_reset(ia_handle* h) {
    { status_reset_k<<<1, 1, 0, h->stream>>>(h->dst); ia::note_launch(); }
    return cuda_fail(cudaGetLastError());
}

// Read the device status once; translate flags to a return code.  For an
// over/under-fill the divergence of both velocity fields at the flagged cell
// decides IA_ERR_DIVERGENCE exactly as reportFillError does (src/advection.jl:151,160).
int status_collect(ia_handle* h, const double* u1, const double* u2, ia_status* out, bool merge) {
    cudaError_t e = cudaMemcpyAsync(h->hst, h->dst, sizeof(DevStatus), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return IA_ERR_CUDA;
    ia_status st;
    if (merge && out) st = *out;
    else std::memset(&st, 0, sizeof(st));
    const int code = translate_fill_status(h->g, *h->hst, u1, u2, st);
    if (out) *out = st;
    return code;
}

int translate_fill_status(const Grid& g, const DevStatus& s, const double* u1, const double* u2, ia_status& st) {
    st.flags |= s.flags & (IA_FLAG_NAN | IA_FLAG_OVERFILL | IA_FLAG_UNDERFILL);
    auto div_at = [&](long long I, double& dsum) -> int {
        double acc[2] = {0.0, 0.0};
        const double* us[2] = {u1, u2};
        for (int k = 0; k < 2; ++k)
            for (int d = 0; d < g.D; ++d) {
                double a = 0, b = 0;
                if (cudaMemcpy(&a, us[k] + d * g.N + I + g.s[d], 8, cudaMemcpyDeviceToHost) != cudaSuccess) return IA_ERR_CUDA;
                if (cudaMemcpy(&b, us[k] + d * g.N + I, 8, cudaMemcpyDeviceToHost) != cudaSuccess) return IA_ERR_CUDA;
                acc[k] += a - b;
            }
        dsum = std::fabs(acc[0]) + std::fabs(acc[1]);
        return IA_OK;
    };
    if (s.flags & IA_FLAG_OVERFILL) {
        st.maxf = ord_dec(s.max_enc);
        st.maxid = (long long)(s.max_key & 0xFFFFFFFFull);
        st.fill_dir = int(s.dir);
        double dv = 0;
        if (u1 && u2 && div_at(st.maxid, dv) == IA_OK && (dv > 10.0 || dv != dv)) st.flags |= IA_FLAG_DIVERGENCE;
    }
    if (s.flags & IA_FLAG_UNDERFILL) {
        st.minf = ord_dec(s.min_enc);
        st.minid = (long long)(s.min_key & 0xFFFFFFFFull);
        st.fill_dir = int(s.dir);
        double dv = 0;
        if (u1 && u2 && div_at(st.minid, dv) == IA_OK && (dv > 10.0 || dv != dv)) st.flags |= IA_FLAG_DIVERGENCE;
    }
    int code = IA_OK;
    if (st.flags & IA_FLAG_NAN) code = IA_ERR_NAN;
    else if (st.flags & IA_FLAG_DIVERGENCE) code = IA_ERR_DIVERGENCE;
    else if (st.flags & (IA_FLAG_OVERFILL | IA_FLAG_UNDERFILL)) code = IA_WARN_FILL;
    else if (st.flags & IA_FLAG_POISSON) code = IA_WARN_NOT_CONVERGED;
    st.code = code;
    return code;
}

// One advect! (src/advection.jl:17-78) or one advectVOF1d! sweep sequence.
int vof_sweep(ia_handle* h, const double* fin, double* fout, const double* u1, const double* u2, double dt, int d,
              bool first, int8_t* cbar, double* rhouf, double tol_rep, int counter, float2* dila) {
    const Grid& g = h->g;
    {
        const int k = 0, counter_base = counter;
        SweepArgs a;
        a.g = g;
        a.d = d;
        a.scheme = h->cfg.normal_scheme;
        a.first = first;
        a.fin = fin;
        a.fout = fout;
        a.u1 = u1 + (long long)a.d * g.N;
        a.u2 = u2 + (long long)a.d * g.N;
        a.cbar = cbar;
        a.rhouf_d = rhouf ? rhouf + (long long)a.d * g.N : nullptr;
        a.h = dt / 2.0;
        a.dt = dt;
        a.lrho = h->cfg.lrho;
        a.one_m_lrho = 1.0 - h->cfg.lrho;
        a.hl = (dt / 2.0) * h->cfg.lrho;
        a.tol_rep = tol_rep;
        a.tol_clean = 10.0 * 2.220446049250313e-16;
        double lim = (dt > 0.0 && std::isfinite(dt)) ? 0.5 / dt : 0.0;
        std::memcpy(&a.ulim, &lim, 8);
        a.list = h->list;
        a.list_count = &h->dst->list_count[(2 * (counter_base + k)) & 31];
        a.flist = h->flist;
        a.flist_count = &h->dst->list_count[(2 * (counter_base + k) + 1) & 31];
        a.flux = h->flux;
        a.vals = h->tmp1;
        a.st = h->dst;
        if (dila) {
            const ff rql = ff_split(0.25 * h->cfg.lrho), rq1 = ff_split(0.25 * (h->cfg.lrho + (1.0 - h->cfg.lrho)));
            a.dila = dila;
            a.rq_l_hi = rql.hi;
            a.rq_l_lo = rql.lo;
            a.rq_1_hi = rq1.hi;
            a.rq_1_lo = rq1.lo;
        }
        int tk = timing_begin(h, TK_VOF_BULK);
        cudaError_t e = vof_sweep_bulk(a, h->stream);
        timing_end(h, tk);
        if (e != cudaSuccess) return IA_ERR_CUDA;
        tk = timing_begin(h, TK_VOF_FACES);
        e = vof_sweep_faces(a, h->stream, h->list_blocks);
        timing_end(h, tk);
        if (e != cudaSuccess) return IA_ERR_CUDA;
        tk = timing_begin(h, TK_VOF_LIST);
        e = vof_sweep_cells(a, h->stream, h->list_blocks);
        if (e == cudaSuccess) e = vof_sweep_scatter(a, h->stream, h->list_blocks);
        timing_end(h, tk);
        if (e != cudaSuccess) return IA_ERR_CUDA;
    }
    return IA_OK;
}

int advect_sweeps(ia_handle* h, double* f, const double* u1, const double* u2, double dt, const int* dirs,
                  int nsweeps, int8_t* cbar, double* rhouf, double tol_rep, bool first_writes_cbar,
                  int counter_base) {
    for (int k = 0; k < nsweeps; ++k) {
        const int rc = vof_sweep(h, f, f, u1, u2, dt, dirs[k], first_writes_cbar && k == 0, cbar, rhouf, tol_rep,
                                 counter_base + k);
        if (rc != IA_OK) return rc;
    }
    return IA_OK;
}

int timing_begin(ia_handle* h, int family) {
    Timing& T = h->timing;
    if (!T.on) return -1;
    const size_t k = T.used;
    if (2 * k + 2 > T.pool.size()) {
        for (int i = 0; i < 2; ++i) {
            cudaEvent_t ev;
            if (cudaEventCreate(&ev) != cudaSuccess) return -1;
            T.pool.push_back(ev);
        }
    }
    if (T.fam.size() <= k) T.fam.resize(k + 1);
    T.fam[k] = family;
    cudaEventRecord(T.pool[2 * k], h->stream);
    T.used = k + 1;
    return int(k);
}

void timing_end(ia_handle* h, int token) {
    if (token < 0) return;
    cudaEventRecord(h->timing.pool[2 * token + 1], h->stream);
}

}  // namespace ia

extern "C" {

int ia_timing(ia_handle* h, int32_t enable, double* ms_out, int64_t* launches_out, int32_t n) {
    if (!h) return IA_ERR_INVALID;
    Timing& T = h->timing;
    if (T.used) {
        if (cudaStreamSynchronize(h->stream) != cudaSuccess) return IA_ERR_CUDA;
        for (size_t k = 0; k < T.used; ++k) {
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, T.pool[2 * k], T.pool[2 * k + 1]) == cudaSuccess) {
                T.ms[T.fam[k]] += ms;
                T.launches[T.fam[k]] += 1;
            }
        }
        T.used = 0;
    }
    for (int i = 0; i < n && i < TK_COUNT; ++i) {
        if (ms_out) ms_out[i] = T.ms[i];
        if (launches_out) launches_out[i] = T.launches[i];
    }
    if (enable >= 0) {
        T.on = enable != 0;
        for (int i = 0; i < TK_COUNT; ++i) {
            T.ms[i] = 0;
            T.launches[i] = 0;
        }
    }
    return IA_OK;
}

int64_t ia_launch_count(void) { return (int64_t)launch_count(); }

const char* ia_error_string(int code) {
    switch (code) {
        case IA_OK: return "ok";
        case IA_ERR_NAN: return "NaN in the volume fraction";
        case IA_ERR_DIVERGENCE: return "velocity divergence exploding at an over/under-filled cell";
        case IA_ERR_UNSUPPORTED: return "unsupported configuration";
        case IA_ERR_INVALID: return "invalid argument or unbound field";
        case IA_ERR_CUDA: return "CUDA runtime error";
        case IA_ERR_NO_DEVICE: return "no CUDA device";
        case IA_ERR_TOO_LARGE: return "grid too large";
        case IA_WARN_FILL: return "volume fraction over/under-filled past tolerance";
        case IA_WARN_NOT_CONVERGED: return "Poisson solve stopped at itmx";
    }
    return "unknown code";
}

int ia_create(const ia_config* cfg, ia_handle** out) {
    if (!cfg || !out) return IA_ERR_INVALID;
    *out = nullptr;
    if (cfg->D != 2 && cfg->D != 3) return IA_ERR_UNSUPPORTED;
    if (cfg->exitBC) return IA_ERR_UNSUPPORTED;
    for (int d = 0; d < cfg->D; ++d)
        if (cfg->N[d] < 2) return IA_ERR_INVALID;
    if (cfg->normal_scheme < 0 || cfg->normal_scheme > IA_NORMAL_XYLIC) return IA_ERR_INVALID;
    if (cfg->limiter < 0 || cfg->limiter > IA_LIMITER_TVDDOWN) return IA_ERR_INVALID;
    if (cfg->poisson_mode < IA_POISSON_FP64 || cfg->poisson_mode > IA_POISSON_LEARNED) return IA_ERR_INVALID;
    if (cfg->poisson_mode == IA_POISSON_LEARNED) {   // the net pools twice in 3D
        if (cfg->D != 3) return IA_ERR_UNSUPPORTED;
        for (int d = 0; d < 3; ++d)
            if (cfg->N[d] % 4 != 0) return IA_ERR_UNSUPPORTED;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return IA_ERR_NO_DEVICE;
    ia_handle* h = new (std::nothrow) ia_handle();
    if (!h) return IA_ERR_INVALID;
    h->cfg = *cfg;
    h->g = make_grid(cfg->D, cfg->perdir, cfg->N);
    // cell offsets within a field are 32-bit signed in the stencil kernels
    if (h->g.N >= (1ll << 31)) { delete h; return IA_ERR_TOO_LARGE; }
    cudaGetDevice(&h->device);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device);
    h->list_blocks = (sms > 0 ? sms : 152) * 8;
    h->stream = nullptr;
    const size_t nb = sizeof(double) * (size_t)h->g.N;
    cudaError_t e = cudaSuccess;
    e = e ? e : cudaMalloc(&h->tmp1, nb);
    e = e ? e : cudaMalloc(&h->list, sizeof(unsigned int) * (size_t)h->g.N);
    e = e ? e : cudaMalloc(&h->flist, sizeof(unsigned int) * (size_t)h->g.N);
    e = e ? e : cudaMalloc(&h->flux, nb);
    e = e ? e : cudaMalloc(&h->dst, sizeof(DevStatus));
    e = e ? e : cudaMalloc(&h->partial, sizeof(double) * 4096);
    e = e ? e : cudaMalloc(&h->dscalar, sizeof(double) * 64);
    e = e ? e : cudaMalloc(&h->cbar_own, (size_t)h->g.N);
    e = e ? e : cudaMallocHost(&h->hst, sizeof(DevStatus));
    if (e != cudaSuccess) {
        ia_destroy(h);
        return IA_ERR_CUDA;
    }
    std::memset(&h->fld, 0, sizeof(h->fld));
    int rc = extra_create(h);
    if (rc != IA_OK) {
        ia_destroy(h);
        return rc;
    }
    *out = h;
    return IA_OK;
}

int ia_destroy(ia_handle* h) {
    if (!h) return IA_OK;
    extra_destroy(h);
    for (cudaEvent_t ev : h->timing.pool) cudaEventDestroy(ev);
    cudaFree(h->tmp1);
    cudaFree(h->list);
    cudaFree(h->flist);
    cudaFree(h->flux);
    cudaFree(h->dst);
    cudaFree(h->partial);
    cudaFree(h->dscalar);
    cudaFree(h->cbar_own);
    if (h->hst) cudaFreeHost(h->hst);
    delete h;
    return IA_OK;
}

int ia_set_stream(ia_handle* h, void* stream) {
    if (!h) return IA_ERR_INVALID;
    h->stream = (cudaStream_t)stream;
    return IA_OK;
}

int ia_bind_fields(ia_handle* h, const ia_fields* fl) {
    if (!h || !fl) return IA_ERR_INVALID;
    h->fld = *fl;
    return IA_OK;
}

int ia_advect_vof(ia_handle* h, double* f, const double* u1, const double* u2, double dt, int64_t n_dt,
                  ia_status* status) {
    if (!h || !f || !u1 || !u2) return IA_ERR_INVALID;
    const int D = h->g.D;
    int dirs[3];
    for (int i = 1; i <= D; ++i) dirs[i - 1] = int((n_dt + i) % D);   // dirO, src/advection.jl:22
    int8_t* cbar = h->fld.cbar ? h->fld.cbar : h->cbar_own;
    int rc = status_reset(h);
    if (rc != IA_OK) return rc;
    rc = advect_sweeps(h, f, u1, u2, dt, dirs, D, cbar, h->fld.rhouf, 10.0 * 2.220446049250313e-16, true, 0);
    if (rc != IA_OK) return rc;
    return status_collect(h, u1, u2, status, false);
}

int ia_reconstruct(ia_handle* h, double* f, double* alpha, double* nhat) {
    if (!h || !f || !alpha || !nhat) return IA_ERR_INVALID;
    return cuda_fail(reconstruct(h->g, h->cfg.normal_scheme, f, alpha, nhat, h->stream));
}

int ia_vof_flux(ia_handle* h, double* fF, const double* f, const double* alpha, const double* nhat, const double* u,
                const double* u0, double dt, int32_t d, double* rhouf) {
    if (!h || !fF || !f || !alpha || !nhat || !u || !u0 || d < 0 || d >= h->g.D) return IA_ERR_INVALID;
    return cuda_fail(vof_flux(h->g, fF, f, alpha, nhat, u, u0, dt, d, rhouf, h->cfg.lrho, h->stream));
}

int ia_apply_vof(ia_handle* h, const double* sdf, double* f, double* alpha, double* nhat) {
    if (!h || !sdf || !f || !alpha || !nhat) return IA_ERR_INVALID;
    return cuda_fail(apply_vof(h->g, sdf, f, alpha, nhat, h->stream));
}

int ia_mass(ia_handle* h, const double* f, double* mass_out) {
    if (!h || !f || !mass_out) return IA_ERR_INVALID;
    cudaError_t e = interior_sum(h->g, f, h->partial, h->dscalar, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(mass_out, h->dscalar, 8, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    return cuda_fail(e);
}

}  // extern "C"
