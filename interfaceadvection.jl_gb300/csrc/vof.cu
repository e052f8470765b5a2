// Direction-split conservative VOF advection (InterfaceAdvection.jl
// src/advection.jl:17-137 with src/normalEstimation.jl and src/PLIC.jl).
//
// One sweep along d maps f_in -> f_out (ping-pong buffers: the update of a
// cell reads f up to two cells away along d, so it cannot run in place).  A
// sweep is two kernels:
//
//  * vof_bulk — one thread per cell of the ghost-inclusive box.  A cell whose
//    three cells along d are all full or all empty, equal to its c̄, and whose
//    face velocities satisfy |u|·δt <= 1/2 leaves the sweep unchanged after
//    cleanWisp!: the face fluxes f·δl and the dilation term cancel to within
//    ~1e-15 < 10 eps.  Those cells are decided with integer compares only
//    (FP64 is slow on this part).  Every other cell is appended to a compacted
//    list.  The kernel also writes the mass flux ρuf[:,d] of faces whose donor
//    cell is full or empty.
//  * vof_list — one thread per listed cell (full warps of interface work):
//    donor-cell reconstruction (normal scheme + PLIC intercept), the PLIC slab
//    volume of each face, the conservative update with the dilation term, the
//    fill-error status, cleanWisp! and the ρuf of the cell's lower face.
//
// Ghost cells are written in the same pass with the value of their
// boundary-condition source cell, so f_out leaves the sweep with BCf! applied
// (src/VOFutil.jl:64-75) and the next sweep reads valid ghosts.
#include <cuda_runtime.h>

#include "ia_core.cuh"
#include "ia_geom.cuh"
#include "vof.cuh"

namespace ia {

namespace {

__device__ __forceinline__ bool abs_le(double v, unsigned long long lim_bits) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFull;
    return b <= lim_bits;   // false for inf / NaN
}

// getVOFFlux! for one face K (lower d-face of cell K), src/advection.jl:113-137.
// Returns the dark-fluid volume fᶠ crossing the face; dl = δt/2 (u1 + u2).
template <int D>
__device__ double face_flux(const SweepArgs& a, long long K, int kd, double& dl) {
    const long long sd = a.g.s[a.d];
    dl = a.h * (a.u1[K] + a.u2[K]);
    if (dl == 0.0) return 0.0;
    const bool pos = dl > 0.0;
    const long long C = pos ? K - sd : K;
    const int cd = pos ? kd - 1 : kd;
    const double fC = a.fin[C];
    const int nd = a.g.n[a.d];
    const bool ghost = (cd == 0) || (cd == nd - 1);
    // α, n̂ of a zero-gradient ghost are never reconstructed: Σ|n̂| = 0 branch
    if (ghost && !a.g.isper(a.d)) return fC * dl;
    if (fC == 0.0 || fC == 1.0) return fC * dl;
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

__device__ __forceinline__ double mass_flux(double dl, double F, double lrho) {
    return dl * lrho + (1.0 - lrho) * F;   // fᶠ2ρuf, src/VOFutil.jl:218
}

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

template <int D, bool FIRST>
__global__ void __launch_bounds__(256) vof_bulk(SweepArgs a) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z;
    const Grid& g = a.g;
    const bool valid = x < g.n[0] && y < g.n[1];
    bool need = false;
    long long O = 0;
    if (valid) {
        O = lin(g, x, y, z);
        const int c[3] = {x, y, z};
        const int sc[3] = {bc_src(g, 0, x), bc_src(g, 1, y), D == 3 ? bc_src(g, 2, z) : 0};
        const long long S = lin(g, sc[0], sc[1], sc[2]);
        const long long sd = g.s[a.d];
        const double fm = a.fin[S - sd], fc = a.fin[S], fp = a.fin[S + sd];
        int cb;
        if (FIRST) {
            a.cbar[O] = (a.fin[O] < 0.5) ? 0 : 1;   // c̄ over every cell, src/advection.jl:40
            cb = (fc < 0.5) ? 0 : 1;
        } else {
            cb = a.cbar[S];
        }
        const double ul = a.u1[S], ur = a.u1[S + sd], vl = a.u2[S], vr = a.u2[S + sd];
        const bool bulk = (fm == fc) && (fc == fp) && (fc == 0.0 || fc == 1.0) && (cb == (fc == 1.0 ? 1 : 0)) &&
                          abs_le(ul, a.ulim) && abs_le(ur, a.ulim) && abs_le(vl, a.ulim) && abs_le(vr, a.ulim);
        need = !bulk;
        double m = 0.0;
        if (a.rhouf_d && in_face_range<D>(g, a.d, c)) {
            const double dl = a.h * (a.u1[O] + a.u2[O]);
            if (dl != 0.0) {
                const bool pos = dl > 0.0;
                const int cd = pos ? c[a.d] - 1 : c[a.d];
                const double fC = a.fin[pos ? O - sd : O];
                const bool zg_ghost = (cd == 0 || cd == g.n[a.d] - 1) && !g.isper(a.d);
                if (zg_ghost || fC == 0.0 || fC == 1.0) m = mass_flux(dl, fC * dl, a.lrho);
                else need = true;
            }
        }
        if (!need) {
            a.fout[O] = (fc == 1.0) ? 1.0 : 0.0;
            if (a.rhouf_d) a.rhouf_d[O] = m;
        }
    }
    warp_append(a.list, a.list_count, valid && need, (unsigned int)O);
}

template <int D, bool FIRST>
__global__ void __launch_bounds__(128) vof_list(SweepArgs a) {
    const unsigned int count = *a.list_count;
    const Grid& g = a.g;
    const long long sd = g.s[a.d];
    for (unsigned int k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
        const long long O = a.list[k];
        int c[3];
        coords_of<D>(g, O, c);
        const int sc[3] = {bc_src(g, 0, c[0]), bc_src(g, 1, c[1]), D == 3 ? bc_src(g, 2, c[2]) : 0};
        const long long S = lin(g, sc[0], sc[1], sc[2]);
        double dl_lo, dl_hi;
        const double F_lo = face_flux<D>(a, S, sc[a.d], dl_lo);
        const double F_hi = face_flux<D>(a, S + sd, sc[a.d] + 1, dl_hi);
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
        a.fout[O] = v;
        if (a.rhouf_d) {
            double m = 0.0;
            if (in_face_range<D>(g, a.d, c)) {
                double dl = dl_lo, F = F_lo;
                if (O != S) F = face_flux<D>(a, O, c[a.d], dl);
                m = (dl == 0.0) ? 0.0 : mass_flux(dl, F, a.lrho);
            }
            a.rhouf_d[O] = m;
        }
    }
}

template <int D, bool FIRST>
void launch_bulk(const SweepArgs& a, cudaStream_t st) {
    dim3 blk(32, 8, 1);
    dim3 grd((a.g.n[0] + 31) / 32, (a.g.n[1] + 7) / 8, a.g.n[2]);
    vof_bulk<D, FIRST><<<grd, blk, 0, st>>>(a);
}

}  // namespace

cudaError_t vof_sweep_bulk(const SweepArgs& a, cudaStream_t st) {
    if (a.g.D == 2) a.first ? launch_bulk<2, true>(a, st) : launch_bulk<2, false>(a, st);
    else a.first ? launch_bulk<3, true>(a, st) : launch_bulk<3, false>(a, st);
    return cudaGetLastError();
}

cudaError_t vof_sweep_list(const SweepArgs& a, cudaStream_t st, int list_blocks) {
    if (a.g.D == 2) {
        if (a.first) vof_list<2, true><<<list_blocks, 128, 0, st>>>(a);
        else vof_list<2, false><<<list_blocks, 128, 0, st>>>(a);
    } else {
        if (a.first) vof_list<3, true><<<list_blocks, 128, 0, st>>>(a);
        else vof_list<3, false><<<list_blocks, 128, 0, st>>>(a);
    }
    return cudaGetLastError();
}

}  // namespace ia
