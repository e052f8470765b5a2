// Direction-split conservative VOF advection (InterfaceAdvection.jl
// src/advection.jl:17-137 with src/normalEstimation.jl and src/PLIC.jl).
//
// One sweep along d updates f in place, like the reference.  Only interface
// cells change; their new values are staged in a compact buffer and written
// back after every read of the old field has finished.  A sweep is four
// kernels:
//
//  * vof_bulk — one thread per cell of the ghost-inclusive box.  A cell whose
//    three cells along d are all full or all empty, equal to its c̄, and whose
//    face velocities satisfy |u|·δt <= 1/2 leaves the sweep unchanged after
//    cleanWisp!: the face fluxes f·δl and the dilation term cancel to within
//    ~1e-15 < 10 eps.  Those cells are decided with integer compares on the
//    IEEE bit patterns only: on GB300 every FP64 instruction, compares
//    included, issues at 1/64 of the FP32 rate, so the bulk path spends FP64
//    only on the mass flux ρuf.  Cells that need the full update go to a cell
//    list; faces whose donor cell must be reconstructed go to a face list.
//  * vof_faces — one thread per listed face: donor reconstruction (normal
//    scheme + PLIC intercept) and the PLIC slab volume, computed once per face
//    and cached; the face's mass flux ρuf.
//  * vof_cells — one thread per listed cell: the conservative update with the
//    dilation term from the two face fluxes, the fill-error status,
//    cleanWisp!, staged in vals[k].
//  * vof_scatter — f[list[k]] = vals[k].
//
// Ghost cells take the value of their boundary-condition source cell in the
// same sweep, so f leaves the sweep with BCf! applied (src/VOFutil.jl:64-75)
// and the next sweep reads valid ghosts.
#include <cuda_runtime.h>

#include "ff.cuh"
#include "ia_core.cuh"
#include "ia_geom.cuh"
#include "vof.cuh"

namespace ia {

namespace {

constexpr unsigned long long ONE_BITS = 0x3FF0000000000000ull;   // 1.0
constexpr unsigned long long ABS_MASK = 0x7FFFFFFFFFFFFFFFull;

__device__ __forceinline__ unsigned long long bits(double v) { return (unsigned long long)__double_as_longlong(v); }
// |v| <= limit, decided on the bit pattern (false for inf / NaN)
__device__ __forceinline__ bool abs_le(unsigned long long b, unsigned long long lim_bits) {
    return (b & ABS_MASK) <= lim_bits;
}
// f ∈ {+0, 1} exactly
__device__ __forceinline__ bool is_bulk(unsigned long long b) { return b == 0ull || b == ONE_BITS; }

__device__ __forceinline__ double mass_flux(double dl, double F, double lrho) {
    return dl * lrho + (1.0 - lrho) * F;   // fᶠ2ρuf, src/VOFutil.jl:218
}

// getVOFFlux! for one face K whose donor needs reconstruction
// (src/advection.jl:113-137); dl = δt/2 (u1 + u2) is passed in.
template <int D>
__device__ double face_flux_recon(const SweepArgs& a, long long K, int kd, double dl) {
    const long long sd = a.g.s[a.d];
    const bool pos = dl > 0.0;
    const long long C = pos ? K - sd : K;
    const int cd = pos ? kd - 1 : kd;
    const double fC = a.fin[C];
    const int nd = a.g.n[a.d];
    const bool ghost = (cd == 0) || (cd == nd - 1);
    long long R = C;   // periodic ghost donors carry their image's reconstruction (BCVOF!)
    if (ghost) R = (cd == 0) ? C + (long long)(nd - 2) * sd : C - (long long)(nd - 2) * sd;
    Stencil S;
    S.f = a.fin;
    S.c = R;
    S.s[0] = a.g.s[0];
    S.s[1] = a.g.s[1];
    S.s[2] = a.g.s[2];
    double n[3];
    interface_normal<D>(a.scheme, S, n);
    double sa = fabs(n[0]) + fabs(n[1]);
    if (D == 3) sa += fabs(n[2]);
    if (sa == 0.0) return fC * dl;
    const double alpha = get_intercept<D>(n, fC);
    const double b = pos ? alpha - n[a.d] * (1.0 - dl) : alpha;
    n[a.d] *= fabs(dl);
    return get_volume_fraction<D>(n, b) * dl;
}

// Does face K (d-coordinate kd) need the donor reconstruction?  Returns false
// and the flux when the donor is full/empty or a zero-gradient ghost (whose
// α, n̂ the reference never reconstructs: the Σ|n̂| = 0 branch).
__device__ __forceinline__ bool face_simple(const SweepArgs& a, long long K, int kd, double& dl, double& F) {
    const long long sd = a.g.s[a.d];
    dl = a.h * (a.u1[K] + a.u2[K]);
    const unsigned long long db = bits(dl);
    if ((db & ABS_MASK) == 0ull) {   // δl == 0: no flux, ρuf untouched
        F = 0.0;
        return true;
    }
    const bool pos = !(db >> 63);
    const long long C = pos ? K - sd : K;
    const int cd = pos ? kd - 1 : kd;
    const double fC = a.fin[C];
    const unsigned long long fb = bits(fC);
    const bool zg_ghost = ((cd == 0) || (cd == a.g.n[a.d] - 1)) && !a.g.isper(a.d);
    if (is_bulk(fb)) {
        F = (fb == ONE_BITS) ? dl : 0.0 * dl;
        return true;
    }
    if (zg_ghost || fC == 0.0 || fC == 1.0) {   // -0, or a mixed zero-gradient ghost donor
        F = fC * dl;
        return true;
    }
    return false;
}

// Mass flux ρuf of face K when its donor is full, empty or a zero-gradient
// ghost: with s = u1 + u2 and δl = s·δt/2 the reference's δl λρ + (1-λρ) fᶠ
// is δl for a full donor and δl λρ for an empty one (two FP64 operations;
// the products are re-associated, a relative change below 1e-15).  Returns
// false when the donor needs reconstruction.
__device__ __forceinline__ bool face_mass_simple(const SweepArgs& a, long long K, int kd, double s, double& m) {
    // s = u1[K] + u2[K]
    const long long sd = a.g.s[a.d];
    const unsigned long long sb = bits(s);
    if ((sb & ABS_MASK) == 0ull) {   // δl == 0: ρuf stays 0
        m = 0.0;
        return true;
    }
    const bool pos = !(sb >> 63);
    const long long C = pos ? K - sd : K;
    const int cd = pos ? kd - 1 : kd;
    const double fC = a.fin[C];
    const unsigned long long fb = bits(fC);
    if (fb == ONE_BITS) { m = a.h * s; return true; }
    if (fb == 0ull) { m = a.hl * s; return true; }
    const bool zg_ghost = ((cd == 0) || (cd == a.g.n[a.d] - 1)) && !a.g.isper(a.d);
    if (zg_ghost || fC == 0.0 || fC == 1.0) {
        const double dl = a.h * s;
        m = dl * a.lrho + a.one_m_lrho * (fC * dl);
        return true;
    }
    return false;
}

// u1[K] + u2[K] for the rare faces whose sum the caller has not formed (out of line: a call is not
// if-converted into the common path)
__device__ __noinline__ double face_sum_cold(const double* u1, const double* u2, long long K) { return u1[K] + u2[K]; }

template <int D>
__device__ __forceinline__ void coords_of(const Grid& g, long long O, int c[3]) {
    c[0] = int(O % g.n[0]);
    const long long r = O / g.n[0];
    c[1] = int(r % g.n[1]);
    c[2] = (D == 3) ? int(r / g.n[1]) : 0;
}

template <int D>
__device__ __forceinline__ bool in_face_range(const Grid& g, int d, const int c[3]) {
#pragma unroll
    for (int e = 0; e < D; ++e) {
        const int hi = (e == d) ? g.n[e] - 1 : g.n[e] - 2;
        if (c[e] < 1 || c[e] > hi) return false;
    }
    return true;
}

__device__ __forceinline__ void warp_append(unsigned int* list, unsigned int* count, bool pred, unsigned int val) {
    const unsigned int mask = __ballot_sync(0xFFFFFFFFu, pred);
    if (!mask) return;
    const int lane = threadIdx.x & 31;   // blocks are 32 wide in x: one warp per row
    const int leader = __ffs(mask) - 1;
    unsigned int base = 0;
    if (lane == leader) base = atomicAdd(count, (unsigned int)__popc(mask));
    base = __shfl_sync(0xFFFFFFFFu, base, leader);
    if (pred) list[base + __popc(mask & ((1u << lane) - 1u))] = val;
}

template <int D, bool FIRST, bool DILA>
__global__ void __launch_bounds__(256) vof_bulk(SweepArgs a) {
    // x in [1, n-2] one cell per lane, so that a row of 32k interior cells fills k warps; the
    // last block column's first warp takes the ghost cells x = 0 and n-1 of the block's 8 rows.
    // Lanes without a cell stay in the warp (the list appends are warp-collective).
    const Grid& g = a.g;
    const bool gcol = blockIdx.x + 1 == gridDim.x;
    const int x = gcol ? ((threadIdx.x & 1) ? g.n[0] - 1 : 0) : 1 + int(blockIdx.x) * 32 + int(threadIdx.x);
    const int y = gcol ? int(blockIdx.y) * 8 + int(threadIdx.x >> 1) : int(blockIdx.y) * 8 + int(threadIdx.y);
    const int z = blockIdx.z;
    const bool valid = (gcol ? (threadIdx.y == 0 && threadIdx.x < 16) : x <= g.n[0] - 2) && y < g.n[1];
    bool need_cell = false, need_face = false;
    long long O = 0;
    if (valid) {
        O = lin(g, x, y, z);
        const int c[3] = {x, y, z};
        const long long S = lin(g, bc_src(g, 0, x), bc_src(g, 1, y), D == 3 ? bc_src(g, 2, z) : 0);
        const long long sd = g.s[a.d];
        const unsigned long long bm = bits(a.fin[S - sd]), bc = bits(a.fin[S]), bp = bits(a.fin[S + sd]);
        int cb;
        if (FIRST) {
            // c̄ = f < 0.5 ? 0 : 1 over every cell (src/advection.jl:40), on the bit pattern
            const unsigned long long bo = bits(a.fin[O]);
            const bool lt_half = ((bo & ABS_MASK) <= 0x7FF0000000000000ull) &&            // not NaN
                                 ((bo >> 63) || bo < 0x3FE0000000000000ull);             // negative or < 0.5
            a.cbar[O] = lt_half ? 0 : 1;
            cb = (bc == ONE_BITS) ? 1 : 0;          // only consulted when bc is bulk
        } else {
            cb = a.cbar[S];
        }
        const bool bulk = (bm == bc) && (bc == bp) && is_bulk(bc) && (cb == (bc == ONE_BITS ? 1 : 0)) &&
                          abs_le(bits(a.u1[S]), a.ulim) && abs_le(bits(a.u1[S + sd]), a.ulim) &&
                          abs_le(bits(a.u2[S]), a.ulim) && abs_le(bits(a.u2[S + sd]), a.ulim);
        need_cell = !bulk;
        double sS = 0.0;   // u1[S] + u2[S]: the dilation difference's and an interior face's mass flux sum
        if (DILA) {
            // the momentum update's dilation term of this (ghost-mapped) cell, on FP32 pairs: c̄ of the
            // source cell (in the first sweep from its fraction, as the c̄ pass above computes it)
            int cs;
            if (FIRST) cs = (((bc & ABS_MASK) <= 0x7FF0000000000000ull) && ((bc >> 63) || bc < 0x3FE0000000000000ull)) ? 0 : 1;
            else cs = cb;
            // the velocity difference in FP64 as (u1 + u2)(S + δd) − (u1 + u2)(S): the second sum is the face
            // mass flux's for an interior cell, so the cell issues two FP64 additions for both instead of
            // four (this pass is bound by its FP64 work), then one split and a pair product
            sS = a.u1[S] + a.u2[S];
            const double du = (a.u1[S + sd] + a.u2[S + sd]) - sS;
            const ff rq = cs ? ff{a.rq_1_hi, a.rq_1_lo} : ff{a.rq_l_hi, a.rq_l_lo};
            const ff dq = ff_mul(rq, ff_split(du));
            a.dila[O] = make_float2(dq.hi, dq.lo);
        }
        // in place a bulk cell keeps its value and only a stale ghost copy needs a write;
        // out of place (the coupled step keeps f_old) every bulk cell is written
        if (bulk && (a.fin != a.fout || ((O != S) && bits(a.fin[O]) != bc)))
            a.fout[O] = (bc == ONE_BITS) ? 1.0 : 0.0;
        if (in_face_range<D>(g, a.d, c)) {
            double m;
            const double sO = DILA ? (O == S ? sS : face_sum_cold(a.u1, a.u2, O)) : a.u1[O] + a.u2[O];
            if (face_mass_simple(a, O, c[a.d], sO, m)) {
                if (a.rhouf_d) a.rhouf_d[O] = m;
            } else {
                need_face = true;
            }
        } else if (a.rhouf_d) {
            a.rhouf_d[O] = 0.0;
        }
    }
    warp_append(a.list, a.list_count, valid && need_cell, (unsigned int)O);
    warp_append(a.flist, a.flist_count, valid && need_face, (unsigned int)O);
}

template <int D>
__global__ void __launch_bounds__(128) vof_faces(SweepArgs a) {
    const unsigned int count = *a.flist_count;
    for (unsigned int k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
        const long long K = a.flist[k];
        int c[3];
        coords_of<D>(a.g, K, c);
        const double dl = a.h * (a.u1[K] + a.u2[K]);
        const double F = face_flux_recon<D>(a, K, c[a.d], dl);
        a.flux[K] = F;
        if (a.rhouf_d) a.rhouf_d[K] = mass_flux(dl, F, a.lrho);
    }
}

template <int D, bool FIRST>
__global__ void __launch_bounds__(128) vof_cells(SweepArgs a) {
    const unsigned int count = *a.list_count;
    const Grid& g = a.g;
    const long long sd = g.s[a.d];
    for (unsigned int k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
        const long long O = a.list[k];
        int c[3];
        coords_of<D>(g, O, c);
        const int sc[3] = {bc_src(g, 0, c[0]), bc_src(g, 1, c[1]), D == 3 ? bc_src(g, 2, c[2]) : 0};
        const long long S = lin(g, sc[0], sc[1], sc[2]);
        double dl, F_lo, F_hi;
        if (!face_simple(a, S, sc[a.d], dl, F_lo)) F_lo = a.flux[S];
        if (!face_simple(a, S + sd, sc[a.d] + 1, dl, F_hi)) F_hi = a.flux[S + sd];
        const double fS = a.fin[S];
        const int cb = FIRST ? ((fS < 0.5) ? 0 : 1) : a.cbar[S];
        const double du = (a.u1[S + sd] - a.u1[S]) + (a.u2[S + sd] - a.u2[S]);
        double v = fS + ((F_lo - F_hi) + double(cb) * du * a.dt / 2.0);
        // reportFillError (src/advection.jl:145-189): judged before cleanWisp!
        if (O == S) {
            if (v != v) {
                atomicOr(&a.st->flags, IA_FLAG_NAN);
            } else if (v - 1.0 > a.tol_rep) {
                atomicOr(&a.st->flags, IA_FLAG_OVERFILL);
                atomicMax(&a.st->max_enc, ord_enc(v));
                const float e = float(v - 1.0);
                atomicMax(&a.st->max_key, ((unsigned long long)__float_as_uint(e) << 32) | (unsigned long long)O);
                a.st->dir = a.d;
            } else if (v < -a.tol_rep) {
                atomicOr(&a.st->flags, IA_FLAG_UNDERFILL);
                atomicMin(&a.st->min_enc, ord_enc(v));
                const float e = float(-v);
                atomicMax(&a.st->min_key, ((unsigned long long)__float_as_uint(e) << 32) | (unsigned long long)O);
                a.st->dir = a.d;
            }
        }
        // cleanWisp! (src/VOFutil.jl:127-136)
        v = (v < a.tol_clean) ? 0.0 : ((v > 1.0 - a.tol_clean) ? 1.0 : v);
        a.vals[k] = v;
    }
}

__global__ void __launch_bounds__(256) vof_scatter(SweepArgs a) {
    const unsigned int count = *a.list_count;
    for (unsigned int k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x)
        a.fout[a.list[k]] = a.vals[k];
}

template <int D, bool FIRST>
void launch_bulk(const SweepArgs& a, cudaStream_t st) {
    dim3 blk(32, 8, 1);
    dim3 grd((a.g.n[0] - 2 + 31) / 32 + 1, (a.g.n[1] + 7) / 8, a.g.n[2]);
    if (a.dila) { vof_bulk<D, FIRST, true><<<grd, blk, 0, st>>>(a); ia::note_launch(); }
    else { vof_bulk<D, FIRST, false><<<grd, blk, 0, st>>>(a); ia::note_launch(); }
}

}  // namespace

cudaError_t vof_sweep_bulk(const SweepArgs& a, cudaStream_t st) {
    if (a.g.D == 2) a.first ? launch_bulk<2, true>(a, st) : launch_bulk<2, false>(a, st);
    else a.first ? launch_bulk<3, true>(a, st) : launch_bulk<3, false>(a, st);
    return cudaGetLastError();
}

cudaError_t vof_sweep_faces(const SweepArgs& a, cudaStream_t st, int list_blocks) {
    if (a.g.D == 2) { vof_faces<2><<<list_blocks, 128, 0, st>>>(a); ia::note_launch(); }
    else { vof_faces<3><<<list_blocks, 128, 0, st>>>(a); ia::note_launch(); }
    return cudaGetLastError();
}

cudaError_t vof_sweep_scatter(const SweepArgs& a, cudaStream_t st, int list_blocks) {
    { vof_scatter<<<list_blocks / 2, 256, 0, st>>>(a); ia::note_launch(); }
    return cudaGetLastError();
}

cudaError_t vof_sweep_cells(const SweepArgs& a, cudaStream_t st, int list_blocks) {
    if (a.g.D == 2) {
        if (a.first) { vof_cells<2, true><<<list_blocks, 128, 0, st>>>(a); ia::note_launch(); }
        else { vof_cells<2, false><<<list_blocks, 128, 0, st>>>(a); ia::note_launch(); }
    } else {
        if (a.first) { vof_cells<3, true><<<list_blocks, 128, 0, st>>>(a); ia::note_launch(); }
        else { vof_cells<3, false><<<list_blocks, 128, 0, st>>>(a); ia::note_launch(); }
    }
    return cudaGetLastError();
}

}  // namespace ia
