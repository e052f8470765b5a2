// Float-float momentum kernels: the CMOM momentum sweep (src/flow.jl:20-57, 212-241), the viscous
// forcing (src/flow.jl:119-153) and the velocity update (src/flow.jl:244-252) of mom.cu with their
// arithmetic on FP32 pairs (ff.cuh) instead of FP64.
//
// The FP64 kernels of mom.cu spend 11 to 33 FP64 operations per cell; GB300 issues FP64 at 1/64 of
// the FP32 rate, so they run at ~80 % FP64-pipe activity and 12-37 % of HBM bandwidth.  Here the
// same formulas, in the same order, run on FP32 pairs (48-bit significands, relative precision
// ~2^-46): every FP64 field value is split into a pair with integer operations when loaded, results
// that leave the momentum chain (ρu, u, the forcing r) are joined back to FP64 with one FP64
// addition each, and the intermediates passed between these kernels (uStar, the face fluxes Φ, the
// viscous fluxes) are stored as pairs (float2, the size of a double).  Full/empty tests, the
// boundary rules and the rare mixed-cell branches (mixed-face densities, viscosities, the SynDRoM
// mass ratio on a mixed donor face) are those of mom.cu: the branch decisions use the same integer
// tests and the rare branches run the same FP64 code.
//
// Differences to the FP64 kernels are rounding-level (a few units of 2^-46 of the operands of each
// operation); they are checked against the FP64 oracle in the step parity tests at 1e-10.
#include <cuda_runtime.h>

#include <cstring>

#include "ff.cuh"
#include "ia_geom.cuh"
#include "mom.cuh"
#include "mom_common.cuh"

namespace ia {

namespace {

// float-float copies of the step constants (MomConsts), the momentum-flux constants (FluxCtx) and the
// pure-phase face viscosities (ViscCtx)
struct MomFF {
    ff lrho, rho1, inv_lrho, inv_rho1;
    ff uBC[3], gvec[3];
};
struct FluxFF {
    ff half_inv_dt, inv_dt, thr_l, thr_1, kl_l, kl_1, sixth;
};
struct ViscFF {
    unsigned long long mu0bits, mu1bits;   // the FP64 pure-phase values get_mu returns
    ff mu_face0, mu_face1;
};

MomFF mom_ff_consts(const MomConsts& k) {
    MomFF q;
    q.lrho = ff_split(k.lrho);
    q.rho1 = ff_split(k.rho1);
    q.inv_lrho = ff_split(k.inv_lrho);
    q.inv_rho1 = ff_split(k.inv_rho1);
    for (int d = 0; d < 3; ++d) {
        q.uBC[d] = ff_split(k.uBC[d]);
        q.gvec[d] = ff_split(k.gvec[d]);
    }
    return q;
}

__device__ __forceinline__ ff ldff(const float2* p) {
    const float2 v = *p;
    return {v.x, v.y};
}
__device__ __forceinline__ void stff(float2* p, ff v) { *p = make_float2(v.hi, v.lo); }

// x / getρ and x · getρ on a face with cell fractions fa, fb (src/VOFutil.jl:176, 198-211)
__device__ __forceinline__ ff div_rho_ff(const MomConsts& k, const MomFF& q, ff v, double fa, double fb) {
    const unsigned long long a = dbits(fa), b = dbits(fb);
    if (a == b && a == 0ull) return ff_mul(v, q.inv_lrho);
    if (a == b && a == kOneBits) return ff_mul(v, q.inv_rho1);
    return ff_split(div_rho_mixed(k.lrho, k.one_m, ff_join(v), fa, fb));
}
__device__ __forceinline__ ff mul_rho_ff(const MomConsts& k, const MomFF& q, ff v, double fa, double fb) {
    const unsigned long long a = dbits(fa), b = dbits(fb);
    if (a == b && a == 0ull) return ff_mul(v, q.lrho);
    if (a == b && a == kOneBits) return ff_mul(v, q.rho1);
    return ff_split(mul_rho_mixed(k.lrho, k.one_m, ff_join(v), fa, fb));
}

// ------------------------------------------------------------------ uStar = BC!(ρu / ρ(f))
// (components unrolled: the boundary value of component i is then a fixed parameter offset)
// a cell with a Dirichlet face or a ghost source for some component: the general rules
template <int D>
__device__ __forceinline__ void ustar_ff_edge(const MomConsts& k, const MomFF& q, const double* __restrict__ rhou,
                                              const double* __restrict__ f, float2* __restrict__ us, int x, int y,
                                              int z, long long O) {
    const Grid& g = k.g;
#pragma unroll
    for (int i = 0; i < D; ++i) {
        int c[3] = {x, y, z};
        ff v;
        if (vel_bc(g, i, c)) {
            v = q.uBC[i];
        } else {
            const long long P = lin3(g, c);
            v = div_rho_ff(k, q, ff_split(rhou[P + i * g.N]), f[P], f[P - g.s[i]]);
        }
        stff(us + O + i * g.N, v);
    }
}
template <int D>
__global__ void ustar_ff_kern(MomConsts k, MomFF q, const double* __restrict__ rhou, const double* __restrict__ f,
                              float2* __restrict__ us) {
    const Grid& g = k.g;
    GCELL_XYZ
    const long long O = lin(g, x, y, z);
    if (x >= 2 && x <= g.n[0] - 2 && y >= 2 && y <= g.n[1] - 2 && (D == 2 || (z >= 2 && z <= g.n[2] - 2))) {
        // no Dirichlet face and no ghost source for any component: every load first
        double r[D], fm[D];
        const double fO = f[O];
#pragma unroll
        for (int i = 0; i < D; ++i) {
            r[i] = rhou[O + i * g.N];
            fm[i] = f[O - g.s[i]];
        }
#pragma unroll
        for (int i = 0; i < D; ++i) stff(us + O + i * g.N, div_rho_ff(k, q, ff_split(r[i]), fO, fm[i]));
        return;
    }
    ustar_ff_edge<D>(k, q, rhou, f, us, x, y, z, O);
}

// BC!(u) at an interior cell (every coordinate in [1, n-2]) keeps the cell's own value, except the normal
// component on the low wall face of a non-periodic dimension (c[i] = 1), which is the Dirichlet constant
__device__ __forceinline__ bool interior_dirichlet(const Grid& g, int i, const int c[3]) {
    return !g.isper(i) && c[i] == 1;
}

// uStar at a ghost cell straight from u and f: ρu at the source P of a non-Dirichlet
// component is mul_rho of u and f there, as u2ρu! forms it (P lies in [1, n-2] in every dimension)
template <int D>
__device__ __forceinline__ void ustar_ff_edge_u(const MomConsts& k, const MomFF& q, const double* __restrict__ u,
                                             const double* __restrict__ f, float2* __restrict__ us, int x, int y,
                                             int z, long long O) {
    const Grid& g = k.g;
#pragma unroll
    for (int i = 0; i < D; ++i) {
        int c[3] = {x, y, z};
        ff v;
        if (vel_bc(g, i, c)) {
            v = q.uBC[i];
        } else {
            const long long P = lin3(g, c);
            const double fP = f[P], fm = f[P - g.s[i]];
            v = div_rho_ff(k, q, ff_split(mul_rho(k, u[P + i * g.N], fP, fm)), fP, fm);
        }
        stff(us + O + i * g.N, v);
    }
}

// copyto!(u⁰,u); copyto!(f⁰,f); u2ρu!(ρu,u⁰,f⁰) in one pass (as stage_start_kern), plus the first sweep's
// uStar = BC!(ρu / ρ(f⁰)) on every cell from the FP64 ρu: the values ustar_ff_kern gives after that pass
template <int D>
__global__ void stage_start_ff_kern(MomConsts k, MomFF q, const double* __restrict__ us, double* __restrict__ ud,
                                    const double* __restrict__ fs, double* __restrict__ fd,
                                    double* __restrict__ rhou, float2* __restrict__ ustar) {
    const Grid& g = k.g;
    GCELL_XYZ
    const long long O = lin(g, x, y, z);
    const double fO = fs[O];
    fd[O] = fO;
    double uv[D];
#pragma unroll
    for (int i = 0; i < D; ++i) {
        uv[i] = us[O + i * g.N];
        if (ud) ud[O + i * g.N] = uv[i];
    }
    if (x < 1 || x > g.n[0] - 2 || y < 1 || y > g.n[1] - 2 || (D == 3 && (z < 1 || z > g.n[2] - 2))) {
        ustar_ff_edge_u<D>(k, q, us, fs, ustar, x, y, z, O);
        return;
    }
    const int c[3] = {x, y, z};
    double fm[D];
#pragma unroll
    for (int i = 0; i < D; ++i) fm[i] = fs[O - g.s[i]];
#pragma unroll
    for (int i = 0; i < D; ++i) {
        const double r = mul_rho(k, uv[i], fO, fm[i]);
        rhou[O + i * g.N] = r;
        stff(ustar + O + i * g.N, interior_dirichlet(g, i, c) ? q.uBC[i] : div_rho_ff(k, q, ff_split(r), fO, fm[i]));
    }
}

// uStar on the ghost cells (some c[e] in {0, n_e - 1}), for a sweep whose interior cells the previous
// sweep's momentum update has written; one thread per cell of the planes bc_plane_cell numbers, the
// interior ones return, and a cell on an edge or corner is written once per plane with the same value
template <int D>
__global__ void ustar_ff_planes(MomConsts k, MomFF q, const double* __restrict__ rhou, const double* __restrict__ f,
                                float2* __restrict__ us) {
    const Grid& g = k.g;
    int c[3];
    if (!bc_plane_cell(g, blockIdx.x * (long long)blockDim.x + threadIdx.x, c) || is_interior(g, c)) return;
    ustar_ff_edge<D>(k, q, rhou, f, us, c[0], c[1], c[2], lin3(g, c));
}

// ------------------------------------------------------------------ limiters (src/flow.jl:5-15)
// Each limiter λ(u, c, d) is returned as its correction m = λ(u, c, d) - c, from δ₁ = c - u and
// δ₂ = d - c: the SynDRoM blend below needs only m (v_d = c + m, c - v_d = -m).
__device__ __forceinline__ ff ff_signed(bool pos, ff v) { return pos ? v : -v; }
// median(a, 0, b): the one of smaller magnitude when a and b share a sign, else 0
__device__ __forceinline__ ff ff_minmod(ff a, ff b) {
    const bool same = (a.hi > 0.0f && b.hi > 0.0f) || (a.hi < 0.0f && b.hi < 0.0f);
    const bool lt = ff_lt(a, b);
    const ff r = (a.hi > 0.0f) == lt ? a : b;
    return same ? r : ff_from(0.0f);
}

template <int LIM>
__device__ __forceinline__ ff limiter_corr_ff(const FluxFF& Q, ff u, ff c, ff d) {
    if (LIM == IA_LIMITER_UPWIND) return ff_from(0.0f);
    const ff d1 = ff_sub(c, u), d2 = ff_sub(d, c);
    if (LIM == IA_LIMITER_MINMOD)   // median((3c - u)/2, c, (c + d)/2) = c + median(δ₁, 0, δ₂)/2
        return ff_scale2(ff_minmod(d1, d2), 0.5f);
    if (LIM == IA_LIMITER_VANALBADA1) {   // c + max(δ₁δ₂, 0)(δ₁ + δ₂)/(δ₁² + δ₂²)/2
        const ff fac = (ff_zero(d1) && ff_zero(d2)) ? ff_from(0.0f)
                                                    : ff_div(ff_add(d1, d2), ff_add(ff_mul(d1, d1), ff_mul(d2, d2)));
        return ff_scale2(ff_mul(ff_max(ff_mul(d1, d2), ff_from(0.0f)), fac), 0.5f);
    }
    if (LIM == IA_LIMITER_SWEBY || LIM == IA_LIMITER_SUPERBEE || LIM == IA_LIMITER_TVDCEN ||
        LIM == IA_LIMITER_TVDDOWN) {
        // c strictly between u and d, else c; s = sign(d - u)
        if (!ff_lt(ff_min(u, d), c) || !ff_lt(c, ff_max(u, d))) return ff_from(0.0f);
        const bool s = ff_pos(ff_sub(d, u));
        const ff cu = ff_signed(s, d1), dc = ff_signed(s, d2);
        ff r;
        if (LIM == IA_LIMITER_TVDCEN) {
            r = ff_min(cu, ff_scale2(dc, 0.5f));
        } else if (LIM == IA_LIMITER_TVDDOWN) {
            r = ff_min(cu, dc);
        } else {
            const float gam = LIM == IA_LIMITER_SWEBY ? 1.5f : 2.0f;
            r = ff_scale2(ff_max(ff_max(ff_from(0.0f), ff_min(ff_mulf(cu, gam), dc)), ff_min(cu, ff_mulf(dc, gam))),
                          0.5f);
        }
        return ff_signed(s, r);
    }
    // Koren: median((7c + d - 2u)/6, c, median(2c - u, c, d)) = c + median((2δ₁ + δ₂)/6, 0, median(δ₁, 0, δ₂))
    const ff tau = ff_mul(ff_add(ff_scale2(d1, 2.0f), d2), Q.sixth);
    return ff_minmod(tau, ff_minmod(d1, d2));
}

// SynDRoM blend Ψ (v_d + l₂ (v_I - v_d)) = Ψ (c + (1 - l₂) m) once l₂ is known (src/flow.jl:37-57)
__device__ __forceinline__ ff blend(ff Psi, ff l2, ff cc, ff m) {
    return ff_mul(Psi, ff_add(cc, ff_mul(ff_sub(ff_from(1.0f), l2), m)));
}

// l₂ = m_out / m_old on a face whose old density m is mixed, or -1 when m_old < m_out
__device__ __noinline__ double l2_from_m(double mOld, double aP, double dt) {
    const double mOut = aP * dt;
    if (dlt(mOld, mOut)) return -1.0;
    return mOut / mOld;
}

template <int LIM>
__device__ ff phiq_inner_ff(const FluxCtx& F, const FluxFF& Q, ff Psi, ff uu, ff cc, ff dd, double fa, double fb) {
    const ff m = limiter_corr_ff<LIM>(Q, uu, cc, dd);
    const ff aP = ff_abs(Psi);
    const unsigned long long a = dbits(fa), b = dbits(fb);
    ff l2;
    if (a == b && (a == 0ull || a == kOneBits)) {
        const bool light = a == 0ull;
        if (ff_lt(light ? Q.thr_l : Q.thr_1, aP)) return ff_mul(Psi, cc);
        l2 = ff_mul(aP, light ? Q.kl_l : Q.kl_1);
    } else {
        const double l = l2_mixed(F, fa, fb, ff_join(aP));
        if (l < 0.0) return ff_mul(Psi, cc);
        l2 = ff_split(l);
    }
    return blend(Psi, l2, cc, m);
}

template <int LIM>
__device__ ff phiq_ff(const FluxCtx& F, const FluxFF& Q, int i, const int cic[3], ff Psi, ff uu, ff cc, ff dd) {
    int c[3] = {cic[0], cic[1], cic[2]};
    if (ff_pos(Psi)) c[F.j] -= 1;                        // IiCell = Ψ>0 ? Ii-δj : Ii
    const ff m = limiter_corr_ff<LIM>(Q, uu, cc, dd);
    const ff aP = ff_abs(Psi);
    double mOld = 0.0;
    const int kind = m_old_kind(F, i, c, mOld);
    ff l2;
    if (kind == 1) {
        if (ff_lt(Q.thr_l, aP)) return ff_mul(Psi, cc);
        l2 = ff_mul(aP, Q.kl_l);
    } else if (kind == 2) {
        if (ff_lt(Q.thr_1, aP)) return ff_mul(Psi, cc);
        l2 = ff_mul(aP, Q.kl_1);
    } else {
        const double l = l2_from_m(mOld, ff_join(aP), F.dt);
        if (l < 0.0) return ff_mul(Psi, cc);
        l2 = ff_split(l);
    }
    return blend(Psi, l2, cc, m);
}

// Ψ = ϕ(i, CI(I,j), ρuf/δt) on a face near a boundary (a BC! face holds u_BC, not ρuf)
__device__ __forceinline__ ff face_psi_ff(const FluxCtx& F, const FluxFF& Q, int ca[3], int cb[3]) {
    double va, vb;
    const bool ba = rraw(F, ca, va), bb = rraw(F, cb, vb);
    const ff a = ff_split(va), b = ff_split(vb);
    if (!ba && !bb) return ff_mul(ff_add(a, b), Q.half_inv_dt);
    return ff_scale2(ff_add(ba ? a : ff_mul(a, Q.inv_dt), bb ? b : ff_mul(b, Q.inv_dt)), 0.5f);
}

// The face fluxes of one cell with every rule: boundary faces, periodic images, mixed donor faces
// (the list kernel's work)
template <int LIM>
__device__ __forceinline__ void momflux_ff_cell(const FluxCtx& F, const FluxFF& Q, const float2* __restrict__ us,
                                                float2* __restrict__ Phi, int x, int y, int z) {
    const Grid& g = F.k.g;
    const int j = F.j;
    int c[3] = {x, y, z};
    bool inner = true;
    for (int e = 0; e < g.D; ++e) {
        const int hi = (e == j) ? g.n[e] - 1 : g.n[e] - 2;
        if (c[e] < 1 || c[e] > hi) return;
        if (c[e] < 3 || c[e] > g.n[e] - 3) inner = false;
    }
    const long long K = lin(g, x, y, z);
    if (inner) {
        // no ghost, wall, periodic-image or boundary-face rule reaches this face's stencil
        const long long sj = g.s[j];
        const ff rK = ff_split(F.rj[K]);
        for (int i = 0; i < g.D; ++i) {
            const long long si = g.s[i];
            const ff Psi = ff_mul(ff_add(rK, ff_split(F.rj[K - si])), Q.half_inv_dt);
            const float2* u = us + i * g.N;
            const bool pos = ff_pos(Psi);
            const ff uu = ldff(u + (pos ? K - 2 * sj : K + sj));
            const ff cc = ldff(u + (pos ? K - sj : K));
            const ff dd = ldff(u + (pos ? K : K - sj));
            const long long P = pos ? K - sj : K;
            stff(Phi + K + i * g.N, phiq_inner_ff<LIM>(F, Q, Psi, uu, cc, dd, F.fold[P], F.fold[P - si]));
        }
        return;
    }
    const bool per = g.isper(j);
    if (per && c[j] == g.n[j] - 1) c[j] = 1;              // periodic upper face = lower face
    const long long Kk = lin3(g, c);
    const int kj = c[j];
    const long long sj = g.s[j];
    const bool lower = kj == 1, upper = !per && kj == g.n[j] - 1;
    for (int i = 0; i < g.D; ++i) {
        int ca[3] = {c[0], c[1], c[2]}, cb[3] = {c[0], c[1], c[2]};
        cb[i] -= 1;
        const ff Psi = face_psi_ff(F, Q, ca, cb);                      // ϕ(i, CI(I,j), ρuf)
        const float2* u = us + i * g.N;
        const bool pos = ff_pos(Psi);
        ff uu, cc, dd;
        if (lower && !per) {               // ϕuL: linear extrapolation below the wall
            if (pos) { cc = ldff(u + Kk - sj); dd = ldff(u + Kk); uu = ff_sub(ff_scale2(cc, 2.0f), dd); }
            else { uu = ldff(u + Kk + sj); cc = ldff(u + Kk); dd = ldff(u + Kk - sj); }
        } else if (lower) {                // ϕuP: periodic image of I-2δj
            if (pos) { uu = ldff(u + Kk + (long long)(g.n[j] - 3 - kj) * sj); cc = ldff(u + Kk - sj); dd = ldff(u + Kk); }
            else { uu = ldff(u + Kk + sj); cc = ldff(u + Kk); dd = ldff(u + Kk - sj); }
        } else if (upper) {                // ϕuR
            if (ff_neg(Psi)) { cc = ldff(u + Kk); dd = ldff(u + Kk - sj); uu = ff_sub(ff_scale2(cc, 2.0f), dd); }
            else { uu = ldff(u + Kk - 2 * sj); cc = ldff(u + Kk - sj); dd = ldff(u + Kk); }
        } else {                           // ϕu
            if (pos) { uu = ldff(u + Kk - 2 * sj); cc = ldff(u + Kk - sj); dd = ldff(u + Kk); }
            else { uu = ldff(u + Kk + sj); cc = ldff(u + Kk); dd = ldff(u + Kk - sj); }
        }
        stff(Phi + K + i * g.N, phiq_ff<LIM>(F, Q, i, c, Psi, uu, cc, dd));
    }
}

// warp-aggregated append of the cells a bulk pass leaves to its list kernel
__device__ __forceinline__ void list_append(unsigned int* list, unsigned int* count, bool want, unsigned int val) {
    const unsigned int bal = __ballot_sync(__activemask(), want);
    if (want) {
        const int lane = int(threadIdx.x + threadIdx.y * blockDim.x) & 31;
        const int leader = __ffs(bal) - 1;
        unsigned int base = 0;
        if (lane == leader) base = atomicAdd(count, unsigned(__popc(bal)));
        base = __shfl_sync(bal, base, leader);
        list[base + __popc(bal & ((1u << lane) - 1u))] = val;
    }
}

// Bulk pass: faces whose stencil no boundary rule reaches and whose donor cells' old fractions are all
// one pure phase (for every component) take the short path below; every other cell goes to the list.
// No out-of-line calls and no local arrays on this path.
// IDX: the type of the cell offsets, int where every vector entry index (3N) fits 32 bits (fewer
// instructions per address in this issue-bound pass), long long otherwise
template <int LIM, class IDX>
__global__ void __launch_bounds__(256, 4) momflux_ff_bulk(FluxCtx F, FluxFF Q, const float2* __restrict__ us,
                                                          float2* __restrict__ Phi, unsigned int* __restrict__ list,
                                                          unsigned int* __restrict__ count) {
    const Grid& g = F.k.g;
    SPLIT_XYZ
    const int j = F.j;
    bool in_range = true, inner = true;
    {
        const int c[3] = {x, y, z};
#pragma unroll
        for (int e = 0; e < 3; ++e) {
            if (e >= g.D) break;
            const int hi = (e == j) ? g.n[e] - 1 : g.n[e] - 2;
            if (c[e] < 1 || c[e] > hi) in_range = false;
            if (c[e] < 3 || c[e] > g.n[e] - 3) inner = false;
        }
    }
    const IDX K = IDX(x) + IDX(y) * IDX(g.s[1]) + IDX(z) * IDX(g.s[2]);
    const IDX N = IDX(g.N);
    bool defer = in_range && !inner;
    if (in_range && inner) {
        // every load first, for both signs of Ψ (the donor row K - δj or K, the upwind stencil
        // K - 2δj .. K or K + δj .. K - δj), so that no load waits for the FP64 Ψ or the pure-phase test
        const IDX sj = IDX(g.s[j]);
        const double rK = F.rj[K];
        const unsigned long long oK = dbits(F.fold[K]), oKj = dbits(F.fold[K - sj]);
        double rI[3];
        unsigned long long oKi[3], oKji[3];
        ff um2[3], um1[3], u00[3], up1[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            if (i >= g.D) break;
            const IDX si = IDX(g.s[i]);
            rI[i] = F.rj[K - si];
            oKi[i] = dbits(F.fold[K - si]);
            oKji[i] = dbits(F.fold[K - sj - si]);
            const float2* u = us + IDX(i) * N;
            um2[i] = ldff(u + K - 2 * sj);
            um1[i] = ldff(u + K - sj);
            u00[i] = ldff(u + K);
            up1[i] = ldff(u + K + sj);
        }
        ff Psi[3];
        unsigned long long ph = 0ull;
        bool pure = true;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            if (i >= g.D) break;
            // Ψ = (ρuf[K] + ρuf[K-δi])/(2δt) in FP64, the reference's two operations, on a pipe this
            // kernel leaves almost idle; then one split
            Psi[i] = ff_split((rK + rI[i]) * F.half_inv_dt);
            const bool pos = ff_pos(Psi[i]);   // donor row P = K - δj (Ψ > 0) or K
            const unsigned long long a = pos ? oKj : oK, b = pos ? oKji[i] : oKi[i];
            if (i == 0) ph = a;
            pure = pure & (a == ph) & (b == ph);
        }
        pure = pure & ((ph == 0ull) | (ph == kOneBits));
        if (!pure) {
            defer = true;
        } else {
            const bool light = ph == 0ull;
            const ff thr = light ? Q.thr_l : Q.thr_1, kl = light ? Q.kl_l : Q.kl_1;
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                if (i >= g.D) break;
                const bool pos = ff_pos(Psi[i]);
                const ff uu = pos ? um2[i] : up1[i];
                const ff cc = pos ? um1[i] : u00[i];
                const ff dd = pos ? u00[i] : um1[i];
                const ff m = limiter_corr_ff<LIM>(Q, uu, cc, dd);
                const ff aP = ff_abs(Psi[i]);
                // above the threshold the face takes Ψ c, which is the blend at l₂ = 1: (1 - 1) m = ±0 and
                // c ± 0 = c exactly for the normalised stored pair c
                const ff l2 = ff_lt(thr, aP) ? ff_from(1.0f) : ff_mul(aP, kl);
                stff(Phi + (K + IDX(i) * N), blend(Psi[i], l2, cc, m));
            }
        }
    }
    list_append(list, count, defer, (unsigned int)K);
}

template <int LIM>
__global__ void __launch_bounds__(128) momflux_ff_list(FluxCtx F, FluxFF Q, const float2* __restrict__ us,
                                                       float2* __restrict__ Phi, const unsigned int* __restrict__ list,
                                                       const unsigned int* __restrict__ count) {
    const unsigned int n = *count;
    for (unsigned int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        int c[3];
        coords3(F.k.g, list[k], c);
        momflux_ff_cell<LIM>(F, Q, us, Phi, c[0], c[1], c[2]);
    }
}

// ------------------------------------------------------------------ ρu += δt (Φ(I) - Φ(I+δj) + uOld ϕ(i,I,ρ̄∂ⱼuⱼ))
// dq = ρ̄∂ⱼuⱼ/2 of every cell (ghosts mapped), written by the sweep's VOF bulk pass, so that
// ϕ(i, I, ρ̄∂ⱼuⱼ) = dq(I) + dq(I-δi); one interior cell per thread, every load issued first.
// With NEXT, also the next sweep's uStar = BC!(ρu / ρ(f_next)) on every interior cell: from the FP64 ρu
// just written, split as ustar_ff_kern splits what it reads, so the values are the same; ustar_ff_planes
// then covers the ghost cells.
template <int D, bool NEXT>
__global__ void __launch_bounds__(256, 4) momupdate_ff_kern(MomConsts k, MomFF q, long long sj,
                                                         const float2* __restrict__ Phi,
                                                         const float2* __restrict__ dq,
                                                         const double* __restrict__ uOld, ff dt,
                                                         double* __restrict__ rhou, const double* __restrict__ fn,
                                                         float2* __restrict__ usn) {
    const Grid& g = k.g;
    ICELL_XYZ
    const long long I = lin(g, x, y, z);
    const ff dI = ldff(dq + I);
    ff dm[D], p0[D], p1[D];
    double uo[D], r0[D], fm[D], fI = 0.0;
#pragma unroll
    for (int i = 0; i < D; ++i) {
        dm[i] = ldff(dq + I - g.s[i]);
        p0[i] = ldff(Phi + I + i * g.N);
        p1[i] = ldff(Phi + I + sj + i * g.N);
        uo[i] = uOld[I + i * g.N];
        r0[i] = rhou[I + i * g.N];
    }
    if (NEXT) {
        fI = fn[I];
#pragma unroll
        for (int i = 0; i < D; ++i) fm[i] = fn[I - g.s[i]];
    }
    const int c[3] = {x, y, z};
#pragma unroll
    for (int i = 0; i < D; ++i) {
        const ff r = ff_add(ff_mul(ff_split(uo[i]), ff_add(dI, dm[i])), ff_sub(p0[i], p1[i]));
        const double rn = ff_join(ff_add(ff_mul(dt, r), ff_split(r0[i])));
        rhou[I + i * g.N] = rn;
        if (NEXT)
            stff(usn + I + i * g.N, interior_dirichlet(g, i, c) ? q.uBC[i] : div_rho_ff(k, q, ff_split(rn), fI, fm[i]));
    }
}

// ------------------------------------------------------------------ viscosity
// the pure-phase values are recognised by their bit patterns (no FP64 comparison)
__device__ __forceinline__ ff mu_ff(const ViscFF& W, double mu) {
    const unsigned long long b = dbits(mu);
    if (b == W.mu0bits) return W.mu_face0;
    if (b == W.mu1bits) return W.mu_face1;
    return ff_split(mu);
}

// viscous fluxes of a cell within two cells of a boundary (general ghost and boundary-face rules),
// out of line so that the bulk path above keeps its own register budget
template <int D>
__device__ __noinline__ void viscflux_ff_edge(const ViscCtx& V, const ViscFF& W, float2* __restrict__ Phi6,
                                             const int c[3], long long K) {
    const Grid& g = V.k.g;
    for (int i = 0; i < D; ++i)
        for (int j = i; j < D; ++j) {
            bool ok = true;
            for (int e = 0; e < D; ++e) {
                const int hi = (e == i || e == j) ? g.n[e] - 1 : g.n[e] - 2;
                if (c[e] < 1 || c[e] > hi) ok = false;
            }
            if (!ok) continue;
            const ff mu = mu_ff(W, get_mu(V, i, j, c));
            const ff sji = ff_sub(ff_split(V.u[K + i * g.N]), ff_split(V.u[K - g.s[j] + i * g.N]));
            const ff sij = ff_sub(ff_split(V.u[K + j * g.N]), ff_split(V.u[K - g.s[i] + j * g.N]));
            stff(Phi6 + pair_index(D, i, j) * g.N + K, -ff_mul(mu, ff_add(sji, sij)));
        }
}

// viscous fluxes of a bulk cell next to the interface: the viscosity of each face or edge from its own
// fractions (get_mu_inner)
template <int D>
__device__ __noinline__ void viscflux_ff_mixed(const ViscCtx& V, const ViscFF& W, float2* __restrict__ Phi6,
                                              const int c[3], long long K) {
    const Grid& g = V.k.g;
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
        for (int j = i; j < D; ++j) {
            const ff mu = mu_ff(W, get_mu_inner(V, i, j, c, K));
            const ff sji = ff_sub(ff_split(V.u[K + i * g.N]), ff_split(V.u[K - g.s[j] + i * g.N]));
            const ff s2 = (i == j) ? ff_scale2(sji, 2.0f)
                                   : ff_add(sji, ff_sub(ff_split(V.u[K + j * g.N]), ff_split(V.u[K - g.s[i] + j * g.N])));
            stff(Phi6 + pair_index(D, i, j) * g.N + K, -ff_mul(mu, s2));
        }
}

// Bulk pass: cells whose faces and edges no wall rule reaches and whose viscosities all read one pure
// phase; every other cell goes to the list (mixed viscosities, wall rules, ghost cells: viscflux_ff_list)
// IDX: int where every vector entry index (6N for the fluxes) fits 32 bits, long long otherwise
template <int D, class IDX>
__global__ void __launch_bounds__(256, sizeof(IDX) == 4 ? 5 : 4) viscflux_ff_bulk(ViscCtx V, ViscFF W, float2* __restrict__ Phi6,
                                                           unsigned int* __restrict__ list,
                                                           unsigned int* __restrict__ count) {
    const Grid& g = V.k.g;
    SPLIT_XYZ
    const IDX K = IDX(x) + IDX(y) * IDX(g.s[1]) + IDX(z) * IDX(g.s[2]);
    const IDX N = IDX(g.N);
    // Cells two or more cells inside a wall dimension, and anywhere in the interior of a periodic one:
    // there get_mu's fface reads f at the face cell and the cell below it, the face cell remapped by
    // face_bc only where its periodic coordinate is 0 (to n-2); every other read is either unmapped or a
    // ghost that holds a bitwise copy of its source.
    const int cc[3] = {x, y, z};
    bool inner = true;
#pragma unroll
    for (int e = 0; e < D; ++e) {
        const bool per = g.isper(e);
        inner = inner && cc[e] >= (per ? 1 : 3) && cc[e] <= g.n[e] - (per ? 2 : 3);
    }
    bool pure = false;
    unsigned long long b0 = 0ull;
    if (inner) {
        // the fractions the D(D+1)/2 viscosities read, with P_k the face cell c - δk as face_bc maps it:
        // face (e, c): K, K - s_e; face (k, c - δk): P_k, P_k - s_k; faces (b, c - δa) and (a, c - δb):
        // P_a, P_a - s_b, P_b, P_b - s_a (every compare evaluated, no short circuit: the loads issue
        // together instead of one after another's compare)
        const double* f = V.f;
        IDX P[D];
#pragma unroll
        for (int k = 0; k < D; ++k)
            P[k] = (g.isper(k) && cc[k] == 1) ? K + IDX(g.n[k] - 3) * IDX(g.s[k]) : K - IDX(g.s[k]);
        b0 = dbits(f[K]);
        bool same = true;
#pragma unroll
        for (int e = 0; e < D; ++e)
            same = same & (dbits(f[K - IDX(g.s[e])]) == b0) & (dbits(f[P[e]]) == b0) & (dbits(f[P[e] - IDX(g.s[e])]) == b0);
#pragma unroll
        for (int a = 0; a < D; ++a)
#pragma unroll
            for (int b = a + 1; b < D; ++b)
                same = same & (dbits(f[P[a] - IDX(g.s[b])]) == b0) & (dbits(f[P[b] - IDX(g.s[a])]) == b0);
        pure = same & ((b0 == 0ull) | (b0 == kOneBits));
    }
    if (pure) {
        const ff mu = b0 == 0ull ? W.mu_face0 : W.mu_face1;
        ff uK[D];
#pragma unroll
        for (int i = 0; i < D; ++i) uK[i] = ff_split(V.u[K + IDX(i) * N]);
#pragma unroll
        for (int i = 0; i < D; ++i)
#pragma unroll
            for (int j = i; j < D; ++j) {
                // ∂ⱼuᵢ + ∂ᵢuⱼ; on the diagonal the two are the same difference
                const ff sji = ff_sub(uK[i], ff_split(V.u[K - IDX(g.s[j]) + IDX(i) * N]));
                const ff s2 = (i == j) ? ff_scale2(sji, 2.0f) : ff_add(sji, ff_sub(uK[j], ff_split(V.u[K - IDX(g.s[i]) + IDX(j) * N])));
                stff(Phi6 + IDX(pair_index(D, i, j)) * N + K, -ff_mul(mu, s2));
            }
    }
    list_append(list, count, !pure, (unsigned int)K);
}

template <int D>
__global__ void __launch_bounds__(128) viscflux_ff_list(ViscCtx V, ViscFF W, float2* __restrict__ Phi6,
                                                        const unsigned int* __restrict__ list,
                                                        const unsigned int* __restrict__ count) {
    const Grid& g = V.k.g;
    const unsigned int n = *count;
    for (unsigned int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const long long K = list[k];
        int c[3];
        coords3(g, K, c);
        bool inner = true;
        for (int e = 0; e < D; ++e)
            if (c[e] < 3 || c[e] > g.n[e] - 3) inner = false;
        if (inner) viscflux_ff_mixed<D>(V, W, Phi6, c, K);
        else viscflux_ff_edge<D>(V, W, Phi6, c, K);
    }
}

template <int D>
__global__ void viscacc_ff_kern(Grid g, const float2* __restrict__ Phi6, double* __restrict__ r) {
    ICELL_XYZ
    const long long I = lin(g, x, y, z);
#pragma unroll
    for (int i = 0; i < D; ++i) {
        ff acc = ff_from(0.0f);
#pragma unroll
        for (int j = 0; j < D; ++j) {
            const float2* P = Phi6 + pair_index(D, i, j) * g.N;
            acc = ff_sub(ff_add(acc, ldff(P + I)), ldff(P + I + g.s[j]));
        }
        r[I + i * g.N] = ff_join(acc);
    }
}

// ------------------------------------------------------------------ updateU! (src/flow.jl:244-252)
template <int D, bool A0>
__global__ void updateu_ff_kern(MomConsts k, MomFF q, double* __restrict__ u, double* __restrict__ rhou,
                                const double* __restrict__ u0, const double* __restrict__ F, ff dt, ff w, ff a,
                                ff dtw, const double* __restrict__ fref, const double* __restrict__ fupd,
                                bool write_rhou) {
    const Grid& g = k.g;
    ICELL_XYZ
    const long long I = lin(g, x, y, z);
    double rv[D], Fv[D], u0v[D], fu[D], fr[D];
    const double fuI = fupd[I], frI = A0 ? 0.0 : fref[I];
#pragma unroll
    for (int i = 0; i < D; ++i) {
        rv[i] = rhou[I + i * g.N];
        Fv[i] = F[I + i * g.N];
        u0v[i] = A0 ? 0.0 : u0[I + i * g.N];
        fu[i] = fupd[I - g.s[i]];
        fr[i] = A0 ? 0.0 : fref[I - g.s[i]];
    }
#pragma unroll
    for (int i = 0; i < D; ++i) {
        ff rn = ff_add(ff_split(rv[i]), ff_mul(ff_split(Fv[i]), dt));
        if (!A0) rn = ff_add(ff_mul(a, mul_rho_ff(k, q, ff_split(u0v[i]), frI, fr[i])), rn);   // u2ρu!(n̂, u⁰, c.f)
        rn = ff_mul(rn, w);
        ff v = div_rho_ff(k, q, rn, fuI, fu[i]);
        if (k.has_g) v = ff_add(ff_mul(dtw, q.gvec[i]), v);
        u[I + i * g.N] = ff_join(v);
        if (write_rhou) rhou[I + i * g.N] = ff_join(rn);
    }
}

// ------------------------------------------------------------------ projection and CFL on pairs
// z = div(u) on interior cells (WaterLily div, the source of myproject!, src/flow.jl:328-347), x *= dt on
// every cell (one FP64 product, as in the FP64 kernel)
template <int D>
__global__ void div_scale_ff_kern(Grid g, const double* __restrict__ u, double* __restrict__ zz, double* __restrict__ xx,
                                  double dt) {
    GCELL_XYZ
    const long long I = lin(g, x, y, z);
    xx[I] *= dt;
    if (x < 1 || x > g.n[0] - 2 || y < 1 || y > g.n[1] - 2 || (D == 3 && (z < 1 || z > g.n[2] - 2))) return;
    double hi[D], lo[D];
#pragma unroll
    for (int d = 0; d < D; ++d) {
        hi[d] = u[I + g.s[d] + d * g.N];
        lo[d] = u[I + d * g.N];
    }
    ff s = ff_sub(ff_split(hi[0]), ff_split(lo[0]));
#pragma unroll
    for (int d = 1; d < D; ++d) s = ff_add(s, ff_sub(ff_split(hi[d]), ff_split(lo[d])));
    zz[I] = ff_join(s);
}

// v truncated to its top 20 significand bits as FP32 (|result| <= |v|, short by less than 2^-20 of
// itself); 0 below the FP32 normal range (where ff_split gives 0 as well), NaN above it
__device__ __forceinline__ float est20(double v) {
    const unsigned h = unsigned(dbits(v) >> 32);
    const int e = int((h >> 20) & 0x7FFu);
    if (e < 897) return 0.0f;
    if (e > 1150) return __uint_as_float(0x7FC00000u);
    return __uint_as_float((h & 0x80000000u) | (unsigned(e - 896) << 23) | ((h & 0xFFFFFu) << 3));
}
__device__ __forceinline__ unsigned long long nonneg_bits_ff(double v) {
    const unsigned long long b = dbits(v);
    return (b == 0x8000000000000000ull) ? 0ull : b;
}
__device__ __forceinline__ unsigned long long warp_umax_ff(unsigned long long v) {
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_down_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    return v;
}

// MPCFL's two maxima (src/flow.jl:262-289) with the per-cell sums on pairs: flux_out Σ max(0,u_hi) +
// max(0,-u_lo) and maxTotalFlux Σ max(|u_lo|,|u_hi|); the terms are selected on the sign / magnitude bits,
// the sums joined to FP64 and reduced as non-negative bit patterns (whole x-rows per block, as cfl_kern)
template <int D>
__global__ void cfl_ff_kern(Grid g, const double* __restrict__ u, unsigned long long* out) {
    __shared__ unsigned long long s1[32], s2[32];
    unsigned long long a1 = 0ull, a2 = 0ull;
    float t1 = 0.0f, t2 = 0.0f;
    const int nxi = g.n[0] - 2, nyi = g.n[1] - 2;
    const int rows = nyi * (D == 3 ? g.n[2] - 2 : 1);
    const int dy = int(gridDim.x) % nyi, dz = int(gridDim.x) / nyi;
    int y = 1 + int(blockIdx.x) % nyi, z = (D == 3 ? 1 : 0) + int(blockIdx.x) / nyi;
    for (int rw = blockIdx.x; rw < rows; rw += gridDim.x, y += dy, z += dz + (y > nyi ? 1 : 0), y -= (y > nyi ? nyi : 0)) {
        for (int x = 1 + threadIdx.x; x <= nxi; x += blockDim.x) {
            const long long I = lin(g, x, y, z);
            double lo[D], hi[D];
#pragma unroll
            for (int i = 0; i < D; ++i) {
                lo[i] = u[I + i * g.N];
                hi[i] = u[I + g.s[i] + i * g.N];
            }
            // FP32 upper bounds of the cell's two sums (terms from the top 20 significand bits, each low
            // by less than 2^-20 of itself; FP32 sums of non-negative terms): the pair sums below run only
            // where a bound is above the largest pair sum this thread has seen (t1, t2 are lower bounds
            // of those), so the maxima are those of every cell's pair sums.  inf and NaN take the exact
            // path (a NaN bound fails every comparison).
            float e1 = 0.0f, e2 = 0.0f;
#pragma unroll
            for (int i = 0; i < D; ++i) {
                const float l = est20(lo[i]), h = est20(hi[i]);
                e1 += fmaxf(h, 0.0f) + fmaxf(-l, 0.0f);
                e2 += fmaxf(fabsf(l), fabsf(h));
            }
            if (!(e1 * 1.0001f <= t1)) {
                ff fo = ff_from(0.0f);
#pragma unroll
                for (int i = 0; i < D; ++i) {
                    const ff flo = ff_split(lo[i]), fhi = ff_split(hi[i]);
                    fo = ff_add(fo, ff_add(ff_pos(fhi) ? fhi : ff_from(0.0f), ff_neg(flo) ? -flo : ff_from(0.0f)));
                }
                const unsigned long long b1 = nonneg_bits_ff(ff_join(fo));
                a1 = b1 > a1 ? b1 : a1;
                t1 = fmaxf(t1, fo.hi * 0.999999f);
            }
            if (!(e2 * 1.0001f <= t2)) {
                ff mt = ff_from(0.0f);
#pragma unroll
                for (int i = 0; i < D; ++i) {
                    const bool lo_big = (dbits(lo[i]) & kAbsMask) >= (dbits(hi[i]) & kAbsMask);
                    mt = ff_add(mt, ff_abs(ff_split(lo_big ? lo[i] : hi[i])));
                }
                const unsigned long long b2 = nonneg_bits_ff(ff_join(mt));
                a2 = b2 > a2 ? b2 : a2;
                t2 = fmaxf(t2, mt.hi * 0.999999f);
            }
        }
    }
    a1 = warp_umax_ff(a1);
    a2 = warp_umax_ff(a2);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) {
        s1[w] = a1;
        s2[w] = a2;
    }
    __syncthreads();
    if (w == 0) {
        const int nw = blockDim.x >> 5;
        a1 = warp_umax_ff(lane < nw ? s1[lane] : 0ull);
        a2 = warp_umax_ff(lane < nw ? s2[lane] : 0ull);
        if (lane == 0) {
            atomicMax(out, a1);
            atomicMax(out + 1, a2);
        }
    }
}

}  // namespace

cudaError_t k_ustar_ff(const MomConsts& k, const double* rhou, const double* f, float2* ustar, cudaStream_t s) {
    if (k.g.D == 3) { ustar_ff_kern<3><<<ggrd(k.g), blk(), 0, s>>>(k, mom_ff_consts(k), rhou, f, ustar); ia::note_launch(); }
    else { ustar_ff_kern<2><<<ggrd(k.g), blk(), 0, s>>>(k, mom_ff_consts(k), rhou, f, ustar); ia::note_launch(); }
    return cudaGetLastError();
}

cudaError_t k_momflux_ff(const MomConsts& k, int j, int limiter, const float2* ustar, const double* rhouf_j,
                         const double* fold, double dt, float2* Phi, unsigned int* list, unsigned int* count,
                         int list_blocks, cudaStream_t s) {
    FluxCtx F;
    F.k = k;
    F.j = j;
    F.lim = limiter;
    F.us = nullptr;
    F.rj = rhouf_j;
    F.fold = fold;
    F.dt = dt;
    F.inv_dt = 1.0 / dt;
    F.half_inv_dt = 0.5 / dt;
    F.thr_l = k.lrho / dt;
    F.thr_1 = k.rho1 / dt;
    F.kl_l = dt * k.inv_lrho;
    F.kl_1 = dt * k.inv_rho1;
    FluxFF Q;
    Q.half_inv_dt = ff_split(F.half_inv_dt);
    Q.inv_dt = ff_split(F.inv_dt);
    Q.thr_l = ff_split(F.thr_l);
    Q.thr_1 = ff_split(F.thr_1);
    Q.kl_l = ff_split(F.kl_l);
    Q.kl_1 = ff_split(F.kl_1);
    Q.sixth = ff_split(1.0 / 6.0);
    const dim3 gr = split_grid(k.g);
    if (cudaMemsetAsync(count, 0, sizeof(unsigned int), s) != cudaSuccess) return cudaGetLastError();
    const bool narrow = !k.wide && 3LL * k.g.N < (1LL << 31);
#define MF_FF(L_)                                                                                         \
    {                                                                                                     \
        if (narrow) momflux_ff_bulk<L_, int><<<gr, blk(), 0, s>>>(F, Q, ustar, Phi, list, count);         \
        else momflux_ff_bulk<L_, long long><<<gr, blk(), 0, s>>>(F, Q, ustar, Phi, list, count);          \
        momflux_ff_list<L_><<<list_blocks, 128, 0, s>>>(F, Q, ustar, Phi, list, count);                  \
        ia::note_launches(2);                                                                             \
    }
    switch (limiter) {
        case IA_LIMITER_UPWIND: MF_FF(IA_LIMITER_UPWIND) break;
        case IA_LIMITER_MINMOD: MF_FF(IA_LIMITER_MINMOD) break;
        case IA_LIMITER_VANALBADA1: MF_FF(IA_LIMITER_VANALBADA1) break;
        case IA_LIMITER_SWEBY: MF_FF(IA_LIMITER_SWEBY) break;
        case IA_LIMITER_SUPERBEE: MF_FF(IA_LIMITER_SUPERBEE) break;
        case IA_LIMITER_TVDCEN: MF_FF(IA_LIMITER_TVDCEN) break;
        case IA_LIMITER_TVDDOWN: MF_FF(IA_LIMITER_TVDDOWN) break;
        default: MF_FF(IA_LIMITER_KOREN) break;
    }
#undef MF_FF
    return cudaGetLastError();
}

cudaError_t k_momupdate_ff(const MomConsts& k, int j, const float2* Phi, const float2* dq, const double* uOld, double dt,
                           double* rhou, const double* fn, float2* us_next, cudaStream_t s) {
    const ff dtf = ff_split(dt);
    const long long sj = k.g.s[j];
    const MomFF q = mom_ff_consts(k);
#define IA_MU(D, NX) momupdate_ff_kern<D, NX><<<igrd(k.g), blk(), 0, s>>>(k, q, sj, Phi, dq, uOld, dtf, rhou, fn, us_next)
    if (k.g.D == 3) { if (us_next) IA_MU(3, true); else IA_MU(3, false); }
    else { if (us_next) IA_MU(2, true); else IA_MU(2, false); }
#undef IA_MU
    ia::note_launch();
    return cudaGetLastError();
}

cudaError_t k_stage_start_ff(const MomConsts& k, const double* us, double* ud, const double* fs, double* fd, double* rhou,
                             float2* ustar, cudaStream_t s) {
    if (k.g.D == 3) stage_start_ff_kern<3><<<ggrd(k.g), blk(), 0, s>>>(k, mom_ff_consts(k), us, ud, fs, fd, rhou, ustar);
    else stage_start_ff_kern<2><<<ggrd(k.g), blk(), 0, s>>>(k, mom_ff_consts(k), us, ud, fs, fd, rhou, ustar);
    ia::note_launch();
    return cudaGetLastError();
}

cudaError_t k_ustar_ff_planes(const MomConsts& k, const double* rhou, const double* f, float2* ustar, cudaStream_t s) {
    const unsigned nb = unsigned((bc_plane_cells(k.g) + 255) / 256);
    if (k.g.D == 3) ustar_ff_planes<3><<<nb, 256, 0, s>>>(k, mom_ff_consts(k), rhou, f, ustar);
    else ustar_ff_planes<2><<<nb, 256, 0, s>>>(k, mom_ff_consts(k), rhou, f, ustar);
    ia::note_launch();
    return cudaGetLastError();
}

cudaError_t k_visc_ff(const MomConsts& k, const double* u, const double* f, double lmu, double mu, float2* Phi6,
                      double* r, unsigned int* list, unsigned int* count, int list_blocks, cudaStream_t s) {
    ViscCtx V;
    V.k = k;
    V.u = u;
    V.f = f;
    V.lmu = lmu;
    V.mu = mu;
    V.ratio = lmu / k.lrho;
    auto lin_prop = [](double sv, double l) { return l + (1.0 - l) * sv; };
    auto mu_at = [&](double sv) {
        const double fac = (sv > 0.5) ? 1.0 : lmu / k.lrho;
        const double a = lin_prop(sv, lmu), b = fac * lin_prop(sv, k.lrho);
        return mu * (b < a ? b : a);
    };
    V.mu_face0 = mu_at(0.0);
    V.mu_face1 = mu_at(1.0);
    ViscFF W;
    std::memcpy(&W.mu0bits, &V.mu_face0, 8);
    std::memcpy(&W.mu1bits, &V.mu_face1, 8);
    W.mu_face0 = ff_split(V.mu_face0);
    W.mu_face1 = ff_split(V.mu_face1);
    const bool narrow = !k.wide && 6LL * k.g.N < (1LL << 31);   // the six flux components' entries in 32 bits
    if (cudaMemsetAsync(count, 0, sizeof(unsigned int), s) != cudaSuccess) return cudaGetLastError();
    if (k.g.D == 3) {
        if (narrow) { viscflux_ff_bulk<3, int><<<split_grid(k.g), blk(), 0, s>>>(V, W, Phi6, list, count); ia::note_launch(); }
        else { viscflux_ff_bulk<3, long long><<<split_grid(k.g), blk(), 0, s>>>(V, W, Phi6, list, count); ia::note_launch(); }
        { viscflux_ff_list<3><<<list_blocks, 128, 0, s>>>(V, W, Phi6, list, count); ia::note_launch(); }
        { viscacc_ff_kern<3><<<igrd(k.g), blk(), 0, s>>>(k.g, Phi6, r); ia::note_launch(); }
    } else {
        if (narrow) { viscflux_ff_bulk<2, int><<<split_grid(k.g), blk(), 0, s>>>(V, W, Phi6, list, count); ia::note_launch(); }
        else { viscflux_ff_bulk<2, long long><<<split_grid(k.g), blk(), 0, s>>>(V, W, Phi6, list, count); ia::note_launch(); }
        { viscflux_ff_list<2><<<list_blocks, 128, 0, s>>>(V, W, Phi6, list, count); ia::note_launch(); }
        { viscacc_ff_kern<2><<<igrd(k.g), blk(), 0, s>>>(k.g, Phi6, r); ia::note_launch(); }
    }
    return cudaGetLastError();
}

cudaError_t k_updateu_ff(const MomConsts& k, double* u, double* rhou, const double* u0, const double* F, double dt,
                         const double* fref, const double* fupd, double w, bool write_rhou, cudaStream_t s) {
    const double a = 1.0 / w - 1.0;
    const MomFF q = mom_ff_consts(k);
    const ff dtf = ff_split(dt), wf = ff_split(w), af = ff_split(a), dtw = ff_split(dt * w);
#define UPD_FF(D_, A0_) \
    { updateu_ff_kern<D_, A0_><<<igrd(k.g), blk(), 0, s>>>(k, q, u, rhou, u0, F, dtf, wf, af, dtw, fref, fupd, write_rhou); ia::note_launch(); }
    if (k.g.D == 3) { if (a == 0.0) UPD_FF(3, true) else UPD_FF(3, false) }
    else { if (a == 0.0) UPD_FF(2, true) else UPD_FF(2, false) }
#undef UPD_FF
    return cudaGetLastError();
}

}  // namespace ia

namespace ia {

cudaError_t k_div_scale_ff(const MomConsts& k, const double* u, double* zz, double* xx, double dt, cudaStream_t s) {
    if (k.g.D == 3) { div_scale_ff_kern<3><<<ggrd(k.g), blk(), 0, s>>>(k.g, u, zz, xx, dt); ia::note_launch(); }
    else { div_scale_ff_kern<2><<<ggrd(k.g), blk(), 0, s>>>(k.g, u, zz, xx, dt); ia::note_launch(); }
    return cudaGetLastError();
}
cudaError_t k_cfl_ff(const MomConsts& k, const double* u, unsigned long long* out2, cudaStream_t s) {
    const long long rows = (long long)(k.g.n[1] - 2) * (k.g.D == 3 ? k.g.n[2] - 2 : 1);
    const int nb = int(rows < 1216 ? rows : 1216);
    if (k.g.D == 3) { cfl_ff_kern<3><<<nb, 256, 0, s>>>(k.g, u, out2); ia::note_launch(); }
    else { cfl_ff_kern<2><<<nb, 256, 0, s>>>(k.g, u, out2); ia::note_launch(); }
    return cudaGetLastError();
}

}  // namespace ia
