// The two-phase time step MPFMomStep! (InterfaceAdvection.jl src/flow.jl:60-109)
// and its C-ABI entry points: the density-weighted RK2 predictor/corrector of
// CMOM momentum advection fused with the VOF sweeps, viscous and surface-tension
// forcing, the velocity update, the variable-density projection and MPCFL.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>

#include "capi_internal.cuh"
#include "mom.cuh"
#include "poisson.cuh"

struct MomScratch {
    double* ustar = nullptr;   // uStar: velocity of the momentum being advected (vector)
    double* Phi = nullptr;     // momentum face fluxes of one sweep (vector)
    double* Phi6 = nullptr;    // viscous face / edge fluxes (D(D+1)/2 scalars)
    double* fb = nullptr;      // face fractions for surface tension (D fields)
    int* slist = nullptr;      // per d, the interior cells with a mixed face fraction (D lists of N)
    unsigned int* scount = nullptr;   // D list lengths
    double* ft1 = nullptr;     // out-of-place VOF sweep buffers
    double* ft2 = nullptr;
    double* dq = nullptr;      // dilation term of the float-float momentum update (N FP32 pairs)
    unsigned int* lcount = nullptr;   // length of the cell list a float-float bulk pass leaves (in slist)
    unsigned long long* cfl = nullptr;   // device max reductions (2)
    unsigned long long* hcfl = nullptr;  // pinned host copy
};

namespace ia {

static MomConsts consts(ia_handle* h) {
    MomConsts k;
    k.g = h->g;
    k.lrho = h->cfg.lrho;
    k.one_m = 1.0 - h->cfg.lrho;
    k.rho1 = k.lrho + k.one_m * 1.0;
    k.inv_lrho = 1.0 / k.lrho;
    k.inv_rho1 = 1.0 / k.rho1;
    for (int d = 0; d < 3; ++d) {
        k.uBC[d] = h->cfg.uBC[d];
        k.gvec[d] = h->cfg.g[d];
    }
    k.has_g = h->cfg.has_g;
    k.wide = h->wide_offsets;
    return k;
}

// float-float momentum arithmetic: chosen with ia_momentum_arith, else by the Poisson mode (the plain
// FP64 mode keeps FP64 kernels throughout)
static bool use_ff(const ia_handle* h) {
    if (h->mom_arith >= 0) return h->mom_arith == IA_ARITH_FF;
    return h->cfg.poisson_mode != IA_POISSON_FP64;
}

int extra_create(ia_handle*) { return IA_OK; }   // momentum / MG scratch is allocated on first use

static int ensure_scratch(ia_handle* h) {
    if (h->mom) return IA_OK;
    MomScratch* m = new MomScratch();
    h->mom = m;
    const size_t N = (size_t)h->g.N, D = (size_t)h->g.D;
    const size_t npair = D * (D + 1) / 2;
    cudaError_t e = cudaSuccess;
    e = e ? e : cudaMalloc(&m->ustar, 8 * N * D);
    e = e ? e : cudaMalloc(&m->Phi, 8 * N * D);
    e = e ? e : cudaMalloc(&m->Phi6, 8 * N * npair);
    e = e ? e : cudaMalloc(&m->fb, 8 * N * D);
    e = e ? e : cudaMalloc(&m->slist, 4 * N * D);
    e = e ? e : cudaMalloc(&m->scount, sizeof(unsigned int) * D);
    e = e ? e : cudaMalloc(&m->ft1, 8 * N);
    e = e ? e : cudaMalloc(&m->ft2, 8 * N);
    e = e ? e : cudaMalloc(&m->dq, 8 * N);
    e = e ? e : cudaMalloc(&m->lcount, sizeof(unsigned int));
    e = e ? e : cudaMalloc(&m->cfl, 16);
    e = e ? e : cudaMallocHost(&m->hcfl, 16);
    if (e != cudaSuccess) return IA_ERR_CUDA;
    cudaMemset(m->Phi, 0, 8 * N * D);
    cudaMemset(m->Phi6, 0, 8 * N * npair);
    return mg_create(h);
}

void extra_destroy(ia_handle* h) {
    mg_destroy(h);
    nn_destroy(h);
    MomScratch* m = h->mom;
    if (!m) return;
    cudaFree(m->ustar);
    cudaFree(m->Phi);
    cudaFree(m->Phi6);
    cudaFree(m->fb);
    cudaFree(m->slist);
    cudaFree(m->scount);
    cudaFree(m->ft1);
    cudaFree(m->ft2);
    cudaFree(m->dq);
    cudaFree(m->lcount);
    cudaFree(m->cfl);
    if (m->hcfl) cudaFreeHost(m->hcfl);
    delete m;
    h->mom = nullptr;
}

// advectfq! → advectVOFρuu! (src/flow.jl:157-232): per direction, uStar = BC!(ρu/ρ(f)),
// the VOF sweep f → f' with its mass flux, the CMOM fluxes and ρu += δt r.
// us_ready: k_stage_start_ff wrote the first sweep's uStar (float-float mode)
static int advect_fq(ia_handle* h, double* f, const double* u1, const double* u2, const double* uOld, double dt,
                     const int* dirs, int counter_base, bool us_ready) {
    const Grid& g = h->g;
    MomScratch* m = h->mom;
    const MomConsts k = consts(h);
    cudaStream_t st = h->stream;
    int8_t* cbar = h->fld.cbar ? h->fld.cbar : h->cbar_own;
    double* seq[4];
    if (g.D == 3) { seq[0] = f; seq[1] = m->ft1; seq[2] = m->ft2; seq[3] = f; }
    else { seq[0] = f; seq[1] = m->ft1; seq[2] = f; }
    const double tol = 10.0 * 2.220446049250313e-16;
    for (int q = 0; q < g.D; ++q) {
        const int d = dirs[q];
        double* fin = seq[q];
        double* fout = seq[q + 1];
        const bool ff = use_ff(h);
        float2* us2 = reinterpret_cast<float2*>(m->ustar);
        float2* Phi2 = reinterpret_cast<float2*>(m->Phi);
        int tk = timing_begin(h, TK_MOM);
        // after the first sweep the previous momentum update wrote uStar on the interior cells
        cudaError_t e = cudaSuccess;
        if (!ff) e = k_ustar(k, h->fld.rhou, fin, m->ustar, st);
        else if (q > 0) e = k_ustar_ff_planes(k, h->fld.rhou, fin, us2, st);
        else if (!us_ready) e = k_ustar_ff(k, h->fld.rhou, fin, us2, st);
        if (e != cudaSuccess) return IA_ERR_CUDA;
        timing_end(h, tk);
        float2* dq2 = ff ? reinterpret_cast<float2*>(m->dq) : nullptr;
        int rc = vof_sweep(h, fin, fout, u1, u2, dt, d, q == 0, cbar, h->fld.rhouf, 10.0 * tol, counter_base + q, dq2);
        if (rc != IA_OK) return rc;
        const double* rj = h->fld.rhouf + (long long)d * g.N;
        tk = timing_begin(h, TK_MOM_FLUX);
        // the surface-tension lists are rebuilt after the sweeps: their buffer holds this pass's list
        unsigned int* lst = reinterpret_cast<unsigned int*>(m->slist);
        e = ff ? k_momflux_ff(k, d, h->cfg.limiter, us2, rj, fin, dt, Phi2, lst, m->lcount, h->list_blocks, st)
               : k_momflux(k, d, h->cfg.limiter, m->ustar, rj, fin, dt, m->Phi, st);
        if (e != cudaSuccess) return IA_ERR_CUDA;
        timing_end(h, tk);
        tk = timing_begin(h, TK_MOM_UPDATE);
        e = ff ? k_momupdate_ff(k, d, Phi2, dq2, uOld, dt, h->fld.rhou, fout, q + 1 < g.D ? us2 : nullptr, st)
               : k_momupdate(k, d, m->Phi, uOld, u1, u2, cbar, dt, h->fld.rhou, st);
        if (e != cudaSuccess) return IA_ERR_CUDA;
        timing_end(h, tk);
    }
    return IA_OK;
}

// viscSurfTenρu! (src/flow.jl:113-117) into the forcing buffer r
static int visc_surften(ia_handle* h, const double* f) {
    const Grid& g = h->g;
    MomScratch* m = h->mom;
    const MomConsts k = consts(h);
    cudaStream_t st = h->stream;
    int tk = timing_begin(h, TK_FORCE);
    cudaError_t e;
    if (h->cfg.mu != 0.0 && use_ff(h))
        e = k_visc_ff(k, h->fld.u, f, h->cfg.lmu, h->cfg.mu, reinterpret_cast<float2*>(m->Phi6), h->fld.force,
                      reinterpret_cast<unsigned int*>(m->slist), m->lcount, h->list_blocks, st);
    else if (h->cfg.mu != 0.0) e = k_visc(k, h->fld.u, f, h->cfg.lmu, h->cfg.mu, m->Phi6, h->fld.force, st);
    else e = k_zero(h->fld.force, g.N * g.D, st);
    if (e != cudaSuccess) return IA_ERR_CUDA;
    // the high x-ghost plane of fᶠ after the last VOF sweep is zero when the x walls' normal velocity is
    // zero (and never read when x is periodic)
    if (h->cfg.eta != 0.0 &&
        k_surften(k, f, nullptr, h->cfg.eta, m->fb, h->fld.force, m->slist, m->scount, st) != cudaSuccess)
        return IA_ERR_CUDA;
    timing_end(h, tk);
    return IA_OK;
}

// updateL! + myproject! (src/flow.jl:254-259, 328-347)
static int project(ia_handle* h, const double* f, double dtp, int* iters, double* resid) {
    const MomConsts k = consts(h);
    cudaStream_t st = h->stream;
    int tk = timing_begin(h, TK_UPDATE);
    if (k_updatel(k, h->fld.mu0, f, st) != cudaSuccess) return IA_ERR_CUDA;
    if ((use_ff(h) ? k_div_scale_ff(k, h->fld.u, h->fld.sigma, h->fld.p, dtp, st)
                   : k_div_scale(k, h->fld.u, h->fld.sigma, h->fld.p, dtp, st)) != cudaSuccess)
        return IA_ERR_CUDA;
    timing_end(h, tk);
    int rc = poisson_solve(h, h->fld.p, h->fld.sigma, h->fld.mu0, h->cfg.poisson_tol, h->cfg.poisson_itmx, iters,
                           resid);
    if (rc != IA_OK && rc != IA_WARN_NOT_CONVERGED) return rc;
    tk = timing_begin(h, TK_UPDATE);
    if (k_correct(k, h->fld.u, h->fld.mu0, h->fld.p, dtp, st) != cudaSuccess) return IA_ERR_CUDA;
    const double zero[3] = {h->cfg.uBC[0], h->cfg.uBC[1], h->cfg.uBC[2]};
    if (k_bc_vel(k, h->fld.u, zero, st) != cudaSuccess) return IA_ERR_CUDA;
    timing_end(h, tk);
    return rc;
}

// MPCFL (src/flow.jl:262-281)
static int mpcfl(ia_handle* h, double* out) {
    MomScratch* m = h->mom;
    const MomConsts k = consts(h);
    cudaStream_t st = h->stream;
    cudaMemsetAsync(m->cfl, 0, 16, st);
    if ((use_ff(h) ? k_cfl_ff(k, h->fld.u, m->cfl, st) : k_cfl(k, h->fld.u, m->cfl, st)) != cudaSuccess)
        return IA_ERR_CUDA;
    cudaMemcpyAsync(m->hcfl, m->cfl, 16, cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return IA_ERR_CUDA;
    double fo, mt;
    std::memcpy(&fo, &m->hcfl[0], 8);
    std::memcpy(&mt, &m->hcfl[1], 8);
    const ia_config& c = h->cfg;
    const double dt_adv = 1.0 / (fo + 5.0 * c.nu);
    const double dt_vof = 1.0 / (2.0 * mt);
    double dt_g = 1.0, dt_v = 1.0, dt_s = 1.0;
    if (c.has_g) {
        double g2 = 0.0;
        for (int i = 0; i < h->g.D; ++i) g2 += c.g[i] * c.g[i];
        dt_g = 1.0 / (2.0 * std::sqrt(g2));
    }
    if (c.mu != 0.0) dt_v = 3.0 / (14.0 * c.mu * std::fmax(1.0, c.lmu / c.lrho));
    if (c.eta != 0.0) dt_s = std::sqrt((1.0 + c.lrho) / (8.0 * M_PI * c.eta));
    double mn = dt_vof;
    for (double v : {dt_adv, dt_g, dt_v, dt_s}) mn = v < mn ? v : mn;
    *out = 0.8 * mn;
    return IA_OK;
}

}  // namespace ia

using namespace ia;

extern "C" {

int ia_mom_step(ia_handle* h, double dt, int64_t n_dt, double t_now, ia_status* status) {
    (void)t_now;
    if (!h) return IA_ERR_INVALID;
    if (ensure_scratch(h) != IA_OK) return IA_ERR_CUDA;
    const ia_fields& F = h->fld;
    if (!F.u || !F.u0 || !F.force || !F.sigma || !F.p || !F.mu0 || !F.f || !F.f0 || !F.rhou || !F.rhouf)
        return IA_ERR_INVALID;
    const Grid& g = h->g;
    const MomConsts k = consts(h);
    cudaStream_t st = h->stream;
    const long long N = g.N, NV = g.N * g.D;
    int dirs[3];
    for (int i = 1; i <= g.D; ++i) dirs[i - 1] = int((n_dt + i) % g.D);   // dirO, src/flow.jl:163
    ia_status S;
    std::memset(&S, 0, sizeof(S));
    // ---- predictor: u(n) → u(n+½) with u(n)
    int tk = timing_begin(h, TK_UPDATE);
    // copyto!(u⁰,u); copyto!(f⁰,f); u2ρu!(ρu,u⁰,f⁰) in one pass
    const bool ff = use_ff(h);
    float2* us2 = reinterpret_cast<float2*>(h->mom->ustar);
    if ((ff ? k_stage_start_ff(k, F.u, F.u0, F.f, F.f0, F.rhou, us2, st)
            : k_stage_start(k, F.u, F.u0, F.f, F.f0, F.rhou, st)) != cudaSuccess)
        return IA_ERR_CUDA;
    timing_end(h, tk);
    int rc = status_reset(h);
    if (rc == IA_OK) rc = advect_fq(h, F.f0, F.u0, F.u, F.u, dt, dirs, 0, ff);
    if (rc != IA_OK) return rc;
    rc = status_collect(h, F.u0, F.u, &S, true);
    if (rc == IA_ERR_NAN || rc == IA_ERR_DIVERGENCE || rc == IA_ERR_CUDA) {
        if (status) *status = S;
        return rc;
    }
    tk = timing_begin(h, TK_UPDATE);
    if (k_average(F.f0, F.f, N, st) != cudaSuccess) return IA_ERR_CUDA;          // f⁰ = (f⁰ + f)/2
    timing_end(h, tk);
    if ((rc = visc_surften(h, F.f0)) != IA_OK) return rc;
    tk = timing_begin(h, TK_UPDATE);
    if ((use_ff(h) ? k_updateu_ff(k, F.u, F.rhou, F.u0, F.force, dt, F.f, F.f0, 0.5, false, st)
                   : k_updateu(k, F.u, F.rhou, F.u0, F.force, dt, F.f, F.f0, 0.5, false, st)) != cudaSuccess)
        return IA_ERR_CUDA;
    if (k_bc_vel(k, F.u, h->cfg.uBC, st) != cudaSuccess) return IA_ERR_CUDA;
    timing_end(h, tk);
    int it0 = 0;
    double r0 = 0.0;
    rc = project(h, F.f0, 0.5 * dt, &it0, &r0);
    if (rc != IA_OK && rc != IA_WARN_NOT_CONVERGED) return rc;
    if (rc == IA_WARN_NOT_CONVERGED) S.flags |= IA_FLAG_POISSON;
    S.poisson_iters[0] = it0;
    S.poisson_resid[0] = r0;
    // ---- corrector: u(n) → u(n+1) with u(n+½)
    tk = timing_begin(h, TK_UPDATE);
    // copyto!(f⁰,f); u2ρu!(ρu,u⁰,f) in one pass
    if ((ff ? k_stage_start_ff(k, F.u0, nullptr, F.f, F.f0, F.rhou, us2, st)
            : k_stage_start(k, F.u0, nullptr, F.f, F.f0, F.rhou, st)) != cudaSuccess)
        return IA_ERR_CUDA;
    timing_end(h, tk);
    rc = status_reset(h);
    if (rc == IA_OK) rc = advect_fq(h, F.f, F.u, F.u, F.u0, dt, dirs, 8, ff);
    if (rc != IA_OK) return rc;
    rc = status_collect(h, F.u, F.u, &S, true);
    if (rc == IA_ERR_NAN || rc == IA_ERR_DIVERGENCE || rc == IA_ERR_CUDA) {
        if (status) *status = S;
        return rc;
    }
    if ((rc = visc_surften(h, F.f)) != IA_OK) return rc;
    // a = 0 for w = 1, so ρu⁰ only enters as 0·ρu⁰; u⁰ takes u(n+½) first (src/flow.jl:100)
    tk = timing_begin(h, TK_UPDATE);
    cudaMemcpyAsync(F.u0, F.u, 8 * NV, cudaMemcpyDeviceToDevice, st);
    if ((use_ff(h) ? k_updateu_ff(k, F.u, F.rhou, F.u0, F.force, dt, F.f, F.f, 1.0, true, st)
                   : k_updateu(k, F.u, F.rhou, F.u0, F.force, dt, F.f, F.f, 1.0, true, st)) != cudaSuccess)
        return IA_ERR_CUDA;
    if (k_bc_vel(k, F.u, h->cfg.uBC, st) != cudaSuccess) return IA_ERR_CUDA;
    timing_end(h, tk);
    int it1 = 0;
    double r1 = 0.0;
    rc = project(h, F.f, dt, &it1, &r1);
    if (rc != IA_OK && rc != IA_WARN_NOT_CONVERGED) return rc;
    if (rc == IA_WARN_NOT_CONVERGED) S.flags |= IA_FLAG_POISSON;
    S.poisson_iters[1] = it1;
    S.poisson_resid[1] = r1;
    double cfl = 0.0;
    tk = timing_begin(h, TK_OTHER);
    rc = mpcfl(h, &cfl);
    timing_end(h, tk);
    if (rc != IA_OK) return rc;
    S.dt_next = cfl < 1.2 * dt ? cfl : 1.2 * dt;                                 // push!(Δt, min(MPCFL, 1.2δt))
    int code = IA_OK;
    if (S.flags & (IA_FLAG_OVERFILL | IA_FLAG_UNDERFILL)) code = IA_WARN_FILL;
    else if (S.flags & IA_FLAG_POISSON) code = IA_WARN_NOT_CONVERGED;
    S.code = code;
    if (status) *status = S;
    return code;
}

int ia_cfl(ia_handle* h, double* dt_out) {
    if (!h || !dt_out || !h->fld.u) return IA_ERR_INVALID;
    if (ensure_scratch(h) != IA_OK) return IA_ERR_CUDA;
    return mpcfl(h, dt_out);
}

int ia_bc_velocity(ia_handle* h, double* a) {
    if (!h || !a) return IA_ERR_INVALID;
    return cuda_fail(k_bc_vel(consts(h), a, h->cfg.uBC, h->stream));
}

int ia_poisson_solve(ia_handle* h, double* x, const double* z, const double* L, double tol, int32_t itmx,
                     int32_t* iters, double* resid) {
    if (!h || !x || !z || !L) return IA_ERR_INVALID;
    if (ensure_scratch(h) != IA_OK) return IA_ERR_CUDA;
    int it = 0;
    double r = 0.0;
    const int rc = poisson_solve(h, x, z, L, tol, itmx, &it, &r);
    if (iters) *iters = it;
    if (resid) *resid = r;
    return rc;
}

int ia_poisson_residual(ia_handle* h, double* r, const double* x, const double* z, const double* L, double* linf) {
    if (!h || !r || !x || !z || !L) return IA_ERR_INVALID;
    return poisson_residual(h, r, x, z, L, linf);
}

int ia_poisson_precond(ia_handle* h, int32_t precond, int32_t inner_max, double inner_rtol) {
    if (!h || precond < IA_PRECOND_HYBRID || precond > IA_PRECOND_VCYCLE || inner_max < 1 ||
        !(inner_rtol > 0.0 && inner_rtol < 1.0))
        return IA_ERR_INVALID;
    // the mixed solver takes only the inner FCG limits (its preconditioner is the V-cycle)
    if (h->cfg.poisson_mode == IA_POISSON_FP64) return IA_ERR_UNSUPPORTED;
    if (h->cfg.poisson_mode == IA_POISSON_MIXED && precond != IA_PRECOND_VCYCLE) return IA_ERR_UNSUPPORTED;
    if (ensure_scratch(h) != IA_OK) return IA_ERR_CUDA;
    h->mg->precond = precond;
    h->mg->inner_max = inner_max;
    h->mg->inner_rtol = inner_rtol;
    return IA_OK;
}

int ia_poisson_mg_params(ia_handle* h, int32_t nu1, int32_t nu2, int32_t nuc) {
    if (!h || nu1 < 1 || nu2 < 0 || nuc < 1 || nu1 > 16 || nu2 > 16 || nuc > 256) return IA_ERR_INVALID;
    if (ensure_scratch(h) != IA_OK) return IA_ERR_CUDA;
    h->mg->nu1 = nu1;
    h->mg->nu2 = nu2;
    h->mg->nuc = nuc;
    return IA_OK;
}

int ia_poisson_mg_relax(ia_handle* h, double omega) {
    if (!h || !(omega > 0.0) || !(omega < 2.0)) return IA_ERR_INVALID;
    if (ensure_scratch(h) != IA_OK) return IA_ERR_CUDA;
    h->mg->omega = omega;
    return IA_OK;
}

int ia_poisson_smoother(ia_handle* h, int32_t kind) {
    if (!h || (kind != IA_SMOOTHER_HALFSWEEP && kind != IA_SMOOTHER_BLOCKED)) return IA_ERR_INVALID;
    if (ensure_scratch(h) != IA_OK) return IA_ERR_CUDA;
    h->mg->smoother = kind;
    return IA_OK;
}

int ia_poisson_coef16(ia_handle* h, int32_t on) {
    if (!h || (on != 0 && on != 1)) return IA_ERR_INVALID;
    if (h->cfg.poisson_mode == IA_POISSON_FP64) return on ? IA_ERR_UNSUPPORTED : IA_OK;
    if (on && !coef16_fits(h->cfg.lrho)) return IA_ERR_UNSUPPORTED;
    if (ensure_scratch(h) != IA_OK) return IA_ERR_CUDA;
    h->mg->coef16 = on;
    return IA_OK;
}

int ia_wide_offsets(ia_handle* h, int32_t on) {
    if (!h || (on != 0 && on != 1)) return IA_ERR_INVALID;
    h->wide_offsets = on;
    return IA_OK;
}

int ia_poisson_mg_fine(ia_handle* h, int32_t nu1, int32_t nu2) {
    if (!h || nu1 < 0 || nu2 < 0 || nu1 > 16 || nu2 > 16) return IA_ERR_INVALID;
    if (ensure_scratch(h) != IA_OK) return IA_ERR_CUDA;
    h->mg->nu1f = nu1;
    h->mg->nu2f = nu2;
    return IA_OK;
}

int ia_poisson_slab_rows(ia_handle* h, int32_t rows) {
    if (!h || rows < 0 || (rows > 0 && rows < 8)) return IA_ERR_INVALID;
    if (ensure_scratch(h) != IA_OK) return IA_ERR_CUDA;
    h->mg->slab_rows = rows;
    return IA_OK;
}

int ia_poisson_stats(ia_handle* h, int64_t* out5) {
    if (!h || !out5) return IA_ERR_INVALID;
    for (int i = 0; i < 5; ++i) out5[i] = h->mg ? h->mg->stats[i] : 0;
    return IA_OK;
}

int ia_project(ia_handle* h, const double* f, double dtp, int32_t* iters, double* resid) {
    if (!h || !f || !h->fld.u || !h->fld.p || !h->fld.sigma || !h->fld.mu0) return IA_ERR_INVALID;
    if (ensure_scratch(h) != IA_OK) return IA_ERR_CUDA;
    int it = 0;
    double r = 0.0;
    const int rc = project(h, f, dtp, &it, &r);
    if (iters) *iters = it;
    if (resid) *resid = r;
    return rc;
}

int ia_advect_momentum(ia_handle* h, double* f, const double* u1, const double* u2, const double* uOld, double dt,
                       int64_t n_dt, ia_status* status) {
    if (!h || !f || !u1 || !u2 || !uOld || !h->fld.rhou || !h->fld.rhouf) return IA_ERR_INVALID;
    if (ensure_scratch(h) != IA_OK) return IA_ERR_CUDA;
    int dirs[3];
    for (int i = 1; i <= h->g.D; ++i) dirs[i - 1] = int((n_dt + i) % h->g.D);
    int rc = status_reset(h);
    if (rc == IA_OK) rc = advect_fq(h, f, u1, u2, uOld, dt, dirs, 0, false);
    if (rc != IA_OK) return rc;
    return status_collect(h, u1, u2, status, false);
}

int ia_surften(ia_handle* h, double* forcing, const double* f, const double* fbuffer, double eta) {
    if (!h || !forcing || !f) return IA_ERR_INVALID;
    if (eta == 0.0) return IA_OK;   // surfTen!(…, η::Nothing) = nothing (src/surfaceTension.jl:7)
    if (ensure_scratch(h) != IA_OK) return IA_ERR_CUDA;
    MomScratch* m = h->mom;
    return cuda_fail(k_surften(consts(h), f, fbuffer, eta, m->fb, forcing, m->slist, m->scount, h->stream));
}

int ia_momentum_arith(ia_handle* h, int32_t kind) {
    if (!h || kind < -1 || kind > IA_ARITH_FF) return IA_ERR_INVALID;
    h->mom_arith = kind;
    return IA_OK;
}

int ia_visc_surften(ia_handle* h, const double* f) {
    if (!h || !f || !h->fld.u || !h->fld.force) return IA_ERR_INVALID;
    if (ensure_scratch(h) != IA_OK) return IA_ERR_CUDA;
    return visc_surften(h, f);
}

}  // extern "C"
