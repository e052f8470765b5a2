// Momentum, forcing and projection kernels of MPFMomStep! (InterfaceAdvection.jl
// src/flow.jl, src/VOFutil.jl, src/surfaceTension.jl) on the reference's
// staggered, ghost-padded FP64 layout.
//
// FP64 issues at 1/64 of the FP32 rate on this part, so the kernels keep FP64
// for the arithmetic the reference does and move everything else off the FP64
// pipe: comparisons, min/max and medians use monotone integer keys of the
// IEEE bit patterns (ia_bc.cuh); full/empty cells take branches whose result
// is a precomputed constant (density λρ or λρ+(1-λρ), their reciprocals,
// face viscosities).  Ghost values are produced by the boundary-condition
// source rules of ia_bc.cuh instead of separate ghost passes.
#include <cuda_runtime.h>

#include "ia_geom.cuh"
#include "mom.cuh"
#include "mom_common.cuh"

namespace ia {

namespace {

// ------------------------------------------------------------------ velocity from momentum
__global__ void ustar_kern(MomConsts k, const double* __restrict__ rhou, const double* __restrict__ f,
                           double* __restrict__ us) {
    const Grid& g = k.g;
    GCELL_XYZ
    const long long O = lin(g, x, y, z);
    for (int i = 0; i < g.D; ++i) {
        int c[3] = {x, y, z};
        if (vel_bc(g, i, c)) {
            us[O + i * g.N] = k.uBC[i];
            continue;
        }
        const long long P = lin3(g, c);
        us[O + i * g.N] = div_rho(k, rhou[P + i * g.N], f[P], f[P - g.s[i]]);
    }
}

__global__ void u2rhou_kern(MomConsts k, double* __restrict__ rhou, const double* __restrict__ u,
                            const double* __restrict__ f) {
    const Grid& g = k.g;
    ICELL_XYZ
    const long long I = lin(g, x, y, z);
    for (int i = 0; i < g.D; ++i) rhou[I + i * g.N] = mul_rho(k, u[I + i * g.N], f[I], f[I - g.s[i]]);
}

// Start of an RK2 stage (src/flow.jl:61, 69 and 89, 92): f_dst = f_src and, when u_dst is given,
// u_dst = u_src over every cell; ρu = u_src · getρ(f_src) on interior cells (u2ρu!).  One pass instead of
// two device copies and a u2ρu! pass that reads them back.
template <int D>
__global__ void stage_start_kern(MomConsts k, const double* __restrict__ us, double* __restrict__ ud,
                                 const double* __restrict__ fs, double* __restrict__ fd, double* __restrict__ rhou) {
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
    if (x < 1 || x > g.n[0] - 2 || y < 1 || y > g.n[1] - 2 || (D == 3 && (z < 1 || z > g.n[2] - 2))) return;
#pragma unroll
    for (int i = 0; i < D; ++i) rhou[O + i * g.N] = mul_rho(k, uv[i], fO, fs[O - g.s[i]]);
}

// BC! at one cell: Dirichlet A[i] on the normal faces, ghost copies elsewhere
__device__ __forceinline__ void bcvel_cell(const Grid& g, double* a, const double A[3], const int c0[3]) {
    const bool inner = is_interior(g, c0);
    const long long O = lin3(g, c0);
    for (int i = 0; i < g.D; ++i) {
        int c[3] = {c0[0], c0[1], c0[2]};
        if (vel_bc(g, i, c)) { a[O + i * g.N] = A[i]; continue; }
        if (inner) continue;
        a[O + i * g.N] = a[lin3(g, c) + i * g.N];
    }
}

// BC! changes only the planes c[e] in {0, 1, n_e - 1} of each dimension (the ghost layers and the
// Dirichlet wall faces): one thread per cell of those planes, instead of a launch over every cell.
// A cell on an edge or corner lies on several planes and is written by each with the same value:
// a written value is A[i] or a copy from a source whose coordinates all lie in [1, n-2] with the
// normal one >= 2 on a wall, a position no thread writes.
__global__ void bcvel_kern(MomConsts k, double* a, double A0, double A1, double A2) {
    const Grid& g = k.g;
    int c[3];
    if (!bc_plane_cell(g, blockIdx.x * (long long)blockDim.x + threadIdx.x, c)) return;
    const double A[3] = {A0, A1, A2};
    bcvel_cell(g, a, A, c);
}

// ------------------------------------------------------------------ limiters (src/flow.jl:5-15)
__device__ __forceinline__ double median3(double a, double b, double c) { return dmax(dmin(a, b), dmin(dmax(a, b), c)); }
__device__ __forceinline__ double sgn(double v) { return okey(v) > 0 ? 1.0 : (okey(v) < 0 ? -1.0 : 0.0); }

__device__ __forceinline__ double limiter(int which, double u, double c, double d) {
    switch (which) {
        case IA_LIMITER_UPWIND: return c;
        case IA_LIMITER_MINMOD: return median3((3.0 * c - u) * 0.5, c, (c + d) * 0.5);
        case IA_LIMITER_VANALBADA1: {
            const double al = c - u, be = d - c;
            const double fac = (dbits(al) << 1) == 0 && (dbits(be) << 1) == 0 ? 0.0 : (al + be) / (al * al + be * be);
            return c + dmax(al * be, 0.0) * fac / 2.0;
        }
        case IA_LIMITER_SWEBY:
        case IA_LIMITER_SUPERBEE: {
            const double gam = which == IA_LIMITER_SWEBY ? 1.5 : 2.0;
            if (!dlt(dmin(u, d), c) || !dlt(c, dmax(u, d))) return c;
            const double s = sgn(d - u);
            return c + s * dmax(dmax(0.0, dmin(s * gam * (c - u), s * (d - c))), dmin(s * (c - u), s * gam * (d - c))) / 2.0;
        }
        case IA_LIMITER_TVDCEN: {
            if (!dlt(dmin(u, d), c) || !dlt(c, dmax(u, d))) return c;
            const double s = sgn(d - u);
            return c + s * dmin(s * (c - u), s * (d - c) / 2.0);
        }
        case IA_LIMITER_TVDDOWN: {
            if (!dlt(dmin(u, d), c) || !dlt(c, dmax(u, d))) return c;
            const double s = sgn(d - u);
            return c + s * dmin(s * (c - u), s * (d - c));
        }
        default:   // Koren
            return median3(fma(-2.0, u, fma(7.0, c, d)) * (1.0 / 6.0), c, median3(fma(2.0, c, -u), c, d));
    }
}

// ------------------------------------------------------------------ CMOM face flux
// Ψ = ϕ(i, CI(I,j), ρuf/δt) = (ρuf[a]/δt + ρuf[b]/δt)/2, one product when neither is a BC face
__device__ __forceinline__ double face_psi(const FluxCtx& F, int ca[3], int cb[3]) {
    double va, vb;
    const bool ba = rraw(F, ca, va), bb = rraw(F, cb, vb);
    if (!ba && !bb) return (va + vb) * F.half_inv_dt;
    return ((ba ? va : va * F.inv_dt) + (bb ? vb : vb * F.inv_dt)) / 2.0;
}

// ϕq (src/flow.jl:37-57) on the upwind triple (uu, cc, dd); cic = coords of the face.
// With v_a = 2v_I - v_d and l₁ = 1 - l₂ the reference's Ψ (v_b + v_d)/2 is Ψ (v_d + l₂ (v_I - v_d)).
template <int LIM>
__device__ double phiq(const FluxCtx& F, int i, const int cic[3], double Psi, double uu, double cc, double dd) {
    int c[3] = {cic[0], cic[1], cic[2]};
    if (okey(Psi) > 0) c[F.j] -= 1;                       // IiCell = Ψ>0 ? Ii-δj : Ii
    const double vd = limiter(LIM, uu, cc, dd);
    const double aP = dabs(Psi);
    double mOld = 0.0, l2;
    const int kind = m_old_kind(F, i, c, mOld);
    if (kind == 1) {
        if (dlt(F.thr_l, aP)) return Psi * cc;
        l2 = aP * F.kl_l;
    } else if (kind == 2) {
        if (dlt(F.thr_1, aP)) return Psi * cc;
        l2 = aP * F.kl_1;
    } else {
        const double mOut = aP * F.dt;
        if (dlt(mOld, mOut)) return Psi * cc;
        l2 = mOut / mOld;
    }
    return Psi * fma(l2, cc - vd, vd);
}

// ϕq for a face far from every boundary: donor old fractions at P and P - δi
template <int LIM>
__device__ __forceinline__ double phiq_inner(const FluxCtx& F, double Psi, double uu, double cc, double dd,
                                             double fa, double fb) {
    const double vd = limiter(LIM, uu, cc, dd);
    const double aP = dabs(Psi);
    const unsigned long long a = dbits(fa), b = dbits(fb);
    double l2;
    if (a == b && (a == 0ull || a == kOneBits)) {
        const bool light = a == 0ull;
        if (dlt(light ? F.thr_l : F.thr_1, aP)) return Psi * cc;
        l2 = aP * (light ? F.kl_l : F.kl_1);
    } else {
        l2 = l2_mixed(F, fa, fb, aP);
        if (l2 < 0.0) return Psi * cc;
    }
    return Psi * fma(l2, cc - vd, vd);
}

template <int LIM>
// 40 registers (six 256-thread blocks per SM) without spills: more warps to cover the FP64 latency
__global__ void __launch_bounds__(256, 6) momflux_kern(FluxCtx F, double* __restrict__ Phi) {
    const Grid& g = F.k.g;
    SPLIT_XYZ
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
        for (int i = 0; i < g.D; ++i) {
            const long long si = g.s[i];
            const double Psi = (F.rj[K] + F.rj[K - si]) * F.half_inv_dt;
            const double* u = F.us + i * g.N;
            const bool pos = okey(Psi) > 0;
            const double uu = pos ? u[K - 2 * sj] : u[K + sj];
            const double cc = pos ? u[K - sj] : u[K];
            const double dd = pos ? u[K] : u[K - sj];
            const long long P = pos ? K - sj : K;
            Phi[K + i * g.N] = phiq_inner<LIM>(F, Psi, uu, cc, dd, F.fold[P], F.fold[P - si]);
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
        const double Psi = face_psi(F, ca, cb);                         // ϕ(i, CI(I,j), ρuf)
        const double* u = F.us + i * g.N;
        const bool pos = okey(Psi) > 0;
        double uu, cc, dd;
        if (lower && !per) {               // ϕuL: linear extrapolation below the wall
            if (pos) { cc = u[Kk - sj]; dd = u[Kk]; uu = 2.0 * cc - dd; }
            else { uu = u[Kk + sj]; cc = u[Kk]; dd = u[Kk - sj]; }
        } else if (lower) {                // ϕuP: periodic image of I-2δj
            if (pos) { uu = u[Kk + (long long)(g.n[j] - 3 - kj) * sj]; cc = u[Kk - sj]; dd = u[Kk]; }
            else { uu = u[Kk + sj]; cc = u[Kk]; dd = u[Kk - sj]; }
        } else if (upper) {                // ϕuR
            if (okey(Psi) < 0) { cc = u[Kk]; dd = u[Kk - sj]; uu = 2.0 * cc - dd; }
            else { uu = u[Kk - 2 * sj]; cc = u[Kk - sj]; dd = u[Kk]; }
        } else {                           // ϕu
            if (pos) { uu = u[Kk - 2 * sj]; cc = u[Kk - sj]; dd = u[Kk]; }
            else { uu = u[Kk + sj]; cc = u[Kk]; dd = u[Kk - sj]; }
        }
        Phi[K + i * g.N] = phiq<LIM>(F, i, c, Psi, uu, cc, dd);
    }
}

// ρ̄∂ⱼuⱼ/2 at a (ghost-mapped) cell: getρ(I,c̄,λρ)(∂(d,I,u)+∂(d,I,u⁰))/4, BCf! ghosts; the
// reference's ϕ(i, I, ρ̄∂ⱼuⱼ) = (d(I) + d(I-δi))/2 is then the plain sum of two of these.
__device__ __forceinline__ double dila_q(const MomConsts& k, double rq_l, double rq_1, int d, int c[3],
                                         const double* u1, const double* u2, const int8_t* cbar) {
    const Grid& g = k.g;
    for (int e = 0; e < g.D; ++e) c[e] = bc_src(g, e, c[e]);
    const long long P = lin3(g, c);
    const long long sd = g.s[d];
    return (cbar[P] ? rq_1 : rq_l) * ((u1[P + sd] - u1[P]) + (u2[P + sd] - u2[P]));
}

// ρu += δt (Φ(I) - Φ(I+δj) + uOld ϕ(i, I, ρ̄∂ⱼuⱼ)).  A block owns a 32 x 8 column of cells
// and marches MU_ZC planes up z; each plane's ρ̄∂ⱼuⱼ/2 values (plus the x-1 / y-1 halo) go to
// shared memory and the previous plane's stay in a register, so every value is computed once
// (4 FP64 ops) instead of once per use (4 uses per cell).
template <int D>
__global__ void __launch_bounds__(256) momupdate_kern(MomConsts k, int j, const double* __restrict__ Phi,
                                                      const double* __restrict__ uOld,
                                                      const double* __restrict__ u1d, const double* __restrict__ u2d,
                                                      const int8_t* __restrict__ cbar, double dt,
                                                      double* __restrict__ rhou) {
    const Grid& g = k.g;
    __shared__ double tile[9][33];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int x0 = 1 + blockIdx.x * 32, y0 = 1 + blockIdx.y * 8;
    const int x = x0 + tx, y = y0 + ty;
    const bool active = x <= g.n[0] - 2 && y <= g.n[1] - 2;
    const double rq_l = 0.25 * k.lrho, rq_1 = 0.25 * k.rho1;
    const int zs = D == 3 ? 1 + int(blockIdx.z) * MU_ZC : 0;
    const int ze = D == 3 ? min(zs + MU_ZC, g.n[2] - 1) : 1;
    double dprev = 0.0;
    if (D == 3 && active) {
        int cm[3] = {x, y, zs - 1};
        dprev = dila_q(k, rq_l, rq_1, j, cm, u1d, u2d, cbar);
    }
    for (int z = zs; z < ze; ++z) {
        for (int l = ty * 32 + tx; l < 9 * 33; l += 256) {
            const int xx = x0 - 1 + l % 33, yy = y0 - 1 + l / 33;
            double v = 0.0;
            if (xx <= g.n[0] - 2 && yy <= g.n[1] - 2) {
                int cc[3] = {xx, yy, z};
                v = dila_q(k, rq_l, rq_1, j, cc, u1d, u2d, cbar);
            }
            tile[l / 33][l % 33] = v;
        }
        __syncthreads();
        if (active) {
            const long long I = lin(g, x, y, z);
            const double dI = tile[ty + 1][tx + 1];
            const double dm[3] = {tile[ty + 1][tx], tile[ty][tx + 1], dprev};
            const long long sj = g.s[j];
#pragma unroll
            for (int i = 0; i < D; ++i) {
                const double r = fma(uOld[I + i * g.N], dI + dm[i], Phi[I + i * g.N] - Phi[I + sj + i * g.N]);
                rhou[I + i * g.N] = fma(dt, r, rhou[I + i * g.N]);
            }
            dprev = dI;
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------ viscosity
template <int D>
// five 256-thread blocks per SM (48 registers; the few spills stay in L1): more warps to cover the
// FP64 latency
__global__ void __launch_bounds__(256, 5) viscflux_kern(ViscCtx V, double* __restrict__ Phi6) {
    const Grid& g = V.k.g;
    SPLIT_XYZ
    const int c[3] = {x, y, z};
    const long long K = lin(g, x, y, z);
    bool inner = true;
#pragma unroll
    for (int e = 0; e < D; ++e)
        if (c[e] < 3 || c[e] > g.n[e] - 3) inner = false;
    if (inner) {
        // every face and edge of this cell is a flux position, no boundary rule applies
#pragma unroll
        for (int i = 0; i < D; ++i)
#pragma unroll
            for (int j = i; j < D; ++j) {
                const double mu = get_mu_inner(V, i, j, c, K);
                const double sji = V.u[K + i * g.N] - V.u[K - g.s[j] + i * g.N];
                const double sij = V.u[K + j * g.N] - V.u[K - g.s[i] + j * g.N];
                Phi6[pair_index(D, i, j) * g.N + K] = -(mu * (sji + sij));
            }
        return;
    }
    for (int i = 0; i < D; ++i)
        for (int j = i; j < D; ++j) {
            bool ok = true;
            for (int e = 0; e < D; ++e) {
                const int hi = (e == i || e == j) ? g.n[e] - 1 : g.n[e] - 2;
                if (c[e] < 1 || c[e] > hi) ok = false;
            }
            if (!ok) continue;
            const double mu = get_mu(V, i, j, c);
            const double sji = V.u[K + i * g.N] - V.u[K - g.s[j] + i * g.N];
            const double sij = V.u[K + j * g.N] - V.u[K - g.s[i] + j * g.N];
            Phi6[pair_index(D, i, j) * g.N + K] = -(mu * (sji + sij));
        }
}

__global__ void viscacc_kern(Grid g, const double* __restrict__ Phi6, double* __restrict__ r) {
    ICELL_XYZ
    const long long I = lin(g, x, y, z);
    for (int i = 0; i < g.D; ++i) {
        double acc = 0.0;
        for (int j = 0; j < g.D; ++j) {
            const double* P = Phi6 + pair_index(g.D, i, j) * g.N;
            acc = (acc + P[I]) - P[I + g.s[j]];
        }
        r[I + i * g.N] = acc;
    }
}

__global__ void zero_kern(double* a, long long n) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
        a[q] = 0.0;
}

// ------------------------------------------------------------------ surface tension
__device__ __forceinline__ bool mixed(double v) {
    const unsigned long long b = dbits(v);
    return b != 0ull && b < kOneBits;   // 0 < v < 1 (sign bit set → huge, excluded)
}

// The reference's surface-tension buffer for direction d at coordinate c0, after surfTen!'s
// `@inside fbuffer[I] = ϕ(d,I,f)` and BCf!(d, fbuffer) (src/surfaceTension.jl:10-11,
// src/VOFutil.jl:76-89).  fbuffer is the cVOF's fᶠ, reused for every d, and BCf!(d, ·) never writes
// the high ghost along a non-periodic d: that position keeps the buffer's previous content.  For
// d > 0 it is the previous direction's value there (whose own ghost rules send the d coordinate to
// n-2; every other coordinate is already mapped); for d = 0 it is the last VOF sweep's flux fᶠ, read
// from prev0 (NULL: zero, which is that flux on the plane whenever the wall's normal velocity is 0).
// (fa + fm)/2 of a face whose two cells differ; out of line so that pure faces, which take fa, issue no
// predicated-off FP64 instructions
__device__ __noinline__ double face_avg(double fa, double fm) { return (fa + fm) / 2.0; }

__device__ __forceinline__ double fbuffer_at(const Grid& g, const double* __restrict__ f, int d, const int c0[3],
                                             const double* __restrict__ prev0) {
    int c[3] = {c0[0], c0[1], c0[2]};
    int dd = d;
    if (face_bc(g, d, c)) {
        if (d == 0) return prev0 ? prev0[lin3(g, c)] : 0.0;
        dd = d - 1;
        face_bc(g, dd, c);
    }
    const long long P = lin3(g, c);
    const double fa = f[P], fm = f[P - g.s[dd]];
    return (dbits(fa) == dbits(fm)) ? fa : face_avg(fa, fm);
}

// fbuffer along every d in one pass over f, and per d the list of interior cells where it is mixed
// (the only cells surften_kern changes), appended one warp at a time
template <int D>
__global__ void fbuffer_kern(MomConsts k, const double* __restrict__ f, const double* __restrict__ prev0,
                             double* __restrict__ fb, int* __restrict__ list, unsigned int* __restrict__ count) {
    const Grid& g = k.g;
    GCELL_XYZ
    const int c0[3] = {x, y, z};
    const bool inner = is_interior(g, c0);
    const long long I = lin(g, x, y, z);
    const int lane = int(threadIdx.x) & 31;
    // interior cells: no ghost or never-written position, the face fractions of this cell directly
    // (the dimension fixed at compile time, so that the D + 1 loads issue before the first list append)
    const bool deep = inner && x <= g.n[0] - 2 && y <= g.n[1] - 2;
    double fI = 0.0, fm[D];
    if (deep) {
        fI = f[I];
#pragma unroll
        for (int d = 0; d < D; ++d) fm[d] = f[I - g.s[d]];
    }
#pragma unroll
    for (int d = 0; d < D; ++d) {
        double v;
        if (deep) {
            v = (dbits(fI) == dbits(fm[d])) ? fI : face_avg(fI, fm[d]);
        } else {
            v = fbuffer_at(g, f, d, c0, prev0);
        }
        fb[d * g.N + I] = v;
        const bool want = inner && mixed(v);
        const unsigned int bal = __ballot_sync(__activemask(), want);
        if (want) {
            const int leader = __ffs(bal) - 1;
            unsigned int base = 0;
            if (lane == leader) base = atomicAdd(count + d, unsigned(__popc(bal)));
            base = __shfl_sync(bal, base, leader);
            list[d * g.N + base + __popc(bal & ((1u << lane) - 1u))] = int(I);
        }
    }
}

// getPopinetHeightAdaptive, monotonic (src/surfaceTension.jl:78-101); axis a, direction sg
__device__ double popinet_height(const Grid& g, const double* fb, const int c0[3], int a, int sg) {
    int c[3] = {c0[0], c0[1], c0[2]};
    double fnow = fb[lin3(g, c)];
    double H = fnow - 0.5;
    bool fin = fnow < 1.0;
    while (!fin || mixed(fnow)) {
        c[a] += sg;
        if (c[a] < 0 || c[a] > g.n[a] - 1) break;
        const double fv = fb[lin3(g, c)];
        fnow = dlt(fnow, fv) ? 0.0 : fv;
        H += fnow;
        if (mixed(fnow)) fin = true;
    }
    c[a] = c0[a];
    fnow = fb[lin3(g, c)];
    fin = fnow > 0.0;
    while (!fin || mixed(fnow)) {
        c[a] -= sg;
        if (c[a] < 0 || c[a] > g.n[a] - 1) break;
        const double fv = fb[lin3(g, c)];
        fnow = dlt(fv, fnow) ? 1.0 : fv;
        H += fnow - 1.0;
        if (mixed(fnow)) fin = true;
    }
    return H;
}

// getCurvature (src/surfaceTension.jl:29-59); md = signed 1-based major direction
__device__ double curvature(const Grid& g, const double* fb, const int c[3], int md) {
    const int a = abs(md) - 1;
    const int sg = md > 0 ? 1 : -1;
    if (g.D == 3) {
        const int am = abs(md);
        const int ix = sg * (am % 3 + 1), iy = (am + 1) % 3 + 1;   // getXYdir
        const int ax = abs(ix) - 1, sx = ix > 0 ? 1 : -1, ay = iy - 1;
        double H[3][3];
        for (int yu = -1; yu <= 1; ++yu)
            for (int xu = -1; xu <= 1; ++xu) {
                int q[3] = {c[0], c[1], c[2]};
                q[ax] += xu * sx;
                q[ay] += yu;
                H[xu + 1][yu + 1] = popinet_height(g, fb, q, a, sg);
            }
        const double filt = 0.2;
        const double Hx = (H[2][1] - H[0][1]) / 2.0, Hy = (H[1][2] - H[1][0]) / 2.0;
        const double Hxx = ((H[2][1] + H[0][1] - 2.0 * H[1][1]) + (H[2][0] + H[0][0] - 2.0 * H[1][0]) * filt +
                            (H[2][2] + H[0][2] - 2.0 * H[1][2]) * filt) / (1.0 + 2.0 * filt);
        const double Hyy = ((H[1][2] + H[1][0] - 2.0 * H[1][1]) + (H[0][2] + H[0][0] - 2.0 * H[0][1]) * filt +
                            (H[2][2] + H[2][0] - 2.0 * H[2][1]) * filt) / (1.0 + 2.0 * filt);
        const double Hxy = (H[2][2] + H[0][0] - H[2][0] - H[0][2]) / 4.0;
        const double q1 = 1.0 + Hx * Hx + Hy * Hy;
        return (Hxx * (1.0 + Hy * Hy) + Hyy * (1.0 + Hx * Hx) - 2.0 * Hxy * Hx * Hy) / sqrt(q1 * q1 * q1);
    }
    const int am = abs(md);
    const int ix = (am == 1) ? -2 * sg : sg;   // getXdir
    const int ax = abs(ix) - 1, sx = ix > 0 ? 1 : -1;
    double H[3];
    for (int xu = -1; xu <= 1; ++xu) {
        int q[3] = {c[0], c[1], c[2]};
        q[ax] += xu * sx;
        H[xu + 1] = popinet_height(g, fb, q, a, sg);
    }
    const double Hx = (H[2] - H[0]) / 2.0, Hxx = (H[2] + H[0] - 2.0 * H[1]);
    const double q1 = 1.0 + Hx * Hx;
    return Hxx / sqrt(q1 * q1 * q1);
}

// surfTen! on the listed cells, one per lane: the interface cells fill whole warps and spread
// over every multiprocessor instead of idling most lanes of the warps that hold them
template <int D>
__global__ void surften_kern(MomConsts k, int d, const double* __restrict__ f, const double* __restrict__ fb,
                             double eta, double* __restrict__ r, const int* __restrict__ list,
                             const unsigned int* __restrict__ count) {
    const Grid& g = k.g;
    const unsigned int n = *count;
    for (unsigned int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const long long I = list[q];
    int c[3];
    coords3(g, I, c);
    Stencil S;
    S.f = fb;
    S.c = I;
    S.s[0] = g.s[0];
    S.s[1] = g.s[1];
    S.s[2] = g.s[2];
    double n[3] = {0.0, 0.0, 0.0};
    normal_columns<D, true>(S, n);                      // getInterfaceNormal_WY!
    const int ia = arg_abs_max<D>(n);
    const int md = signbit(n[ia]) ? -(ia + 1) : (ia + 1);
    const double kap = curvature(g, fb, c, md);
    r[I + d * g.N] += eta * kap * -(f[I] - f[I - g.s[d]]);
    }
}

// ------------------------------------------------------------------ update, L, projection
// A0: a = 0 (the corrector, w = 1), where a·ρu⁰ only adds a zero: ρu⁰ is then not formed
template <bool A0>
__global__ void updateu_kern(MomConsts k, double* __restrict__ u, double* __restrict__ rhou,
                             const double* __restrict__ u0, const double* __restrict__ F, double dt,
                             const double* __restrict__ fref, const double* __restrict__ fupd, double w, double a,
                             bool write_rhou) {
    const Grid& g = k.g;
    ICELL_XYZ
    const long long I = lin(g, x, y, z);
    for (int i = 0; i < g.D; ++i) {
        const long long q = I + i * g.N;
        double rn;
        if (A0) {
            rn = (rhou[q] + F[q] * dt) * w;
        } else {
            const double rho0 = mul_rho(k, u0[q], fref[I], fref[I - g.s[i]]);   // u2ρu!(n̂, u⁰, c.f)
            rn = (a * rho0 + rhou[q] + F[q] * dt) * w;
        }
        double v = div_rho(k, rn, fupd[I], fupd[I - g.s[i]]);
        if (k.has_g) v = (dt * w) * k.gvec[i] + v;
        u[q] = v;
        if (write_rhou) rhou[q] = rn;
    }
}

template <int D>
__global__ void updatel_kern(MomConsts k, double* __restrict__ mu0, const double* __restrict__ f) {
    const Grid& g = k.g;
    GCELL_XYZ
    const long long O = lin(g, x, y, z);
    if (x >= 2 && x <= g.n[0] - 2 && y >= 2 && y <= g.n[1] - 2 && (D == 2 || (z >= 2 && z <= g.n[2] - 2))) {
        // no boundary rule: every load first
        const double fo = f[O];
        double fm[D];
#pragma unroll
        for (int i = 0; i < D; ++i) fm[i] = f[O - g.s[i]];
#pragma unroll
        for (int i = 0; i < D; ++i) mu0[O + i * g.N] = div_rho(k, 1.0, fo, fm[i]);
        return;
    }
    for (int i = 0; i < D; ++i) {
        int c[3] = {x, y, z};
        if (vel_bc(g, i, c)) { mu0[O + i * g.N] = 0.0; continue; }
        const long long P = lin3(g, c);
        mu0[O + i * g.N] = div_rho(k, 1.0, f[P], f[P - g.s[i]]);
    }
}

__global__ void div_scale_kern(Grid g, const double* __restrict__ u, double* __restrict__ zz,
                               double* __restrict__ xx, double dt) {
    GCELL_XYZ
    const long long I = lin(g, x, y, z);
    xx[I] *= dt;
    const int c[3] = {x, y, z};
    if (!is_interior(g, c)) return;
    double s = 0.0;
    for (int d = 0; d < g.D; ++d) s += u[I + g.s[d] + d * g.N] - u[I + d * g.N];
    zz[I] = s;
}

// u -= L ∂x on interior cells (the dimension fixed at compile time: every load issued first, no
// dynamically indexed grid strides)
template <int D>
__global__ void correct_kern(Grid g, double* __restrict__ u, const double* __restrict__ L,
                             const double* __restrict__ xx) {
    ICELL_XYZ
    const long long I = lin(g, x, y, z);
    const double xI = xx[I];
    double uu[D], ll[D], xm[D];
#pragma unroll
    for (int i = 0; i < D; ++i) {
        uu[i] = u[I + i * g.N];
        ll[i] = L[I + i * g.N];
        xm[i] = xx[I - g.s[i]];
    }
#pragma unroll
    for (int i = 0; i < D; ++i) u[I + i * g.N] = uu[i] - ll[i] * (xI - xm[i]);
}

__global__ void scale_kern(double* a, long long n, double s) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
        a[q] *= s;
}

__global__ void average_kern(double* a, const double* b, long long n) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
        a[q] = (a[q] + b[q]) / 2.0;
}

__device__ __forceinline__ unsigned long long nonneg_bits(double v) {
    const unsigned long long b = dbits(v);
    return (b == 0x8000000000000000ull) ? 0ull : b;
}

// -u with the sign bit flipped (no FP64 instruction)
__device__ __forceinline__ double dneg(double v) { return __longlong_as_double(__double_as_longlong(v) ^ (1ll << 63)); }

__device__ __forceinline__ unsigned long long warp_umax(unsigned long long v) {
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_down_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    return v;
}

// max over interior cells of WaterLily flux_out (Σ max(0,u_hi) + max(0,-u_lo)) and of
// maxTotalFlux (Σ max(|u_lo|,|u_hi|), src/flow.jl:283-289), as non-negative FP64 bit patterns;
// whole x-rows per block, warp-shuffle maxima
__global__ void cfl_kern(Grid g, const double* __restrict__ u, unsigned long long* out) {
    __shared__ unsigned long long s1[32], s2[32];
    unsigned long long a1 = 0ull, a2 = 0ull;
    const int nxi = g.n[0] - 2, nyi = g.n[1] - 2;
    const int rows = nyi * (g.D == 3 ? g.n[2] - 2 : 1);
    // rows b, b + G, ...: (y, z) advance incrementally
    const int dy = int(gridDim.x) % nyi, dz = int(gridDim.x) / nyi;
    int y = 1 + int(blockIdx.x) % nyi, z = (g.D == 3 ? 1 : 0) + int(blockIdx.x) / nyi;
    for (int rw = blockIdx.x; rw < rows; rw += gridDim.x, y += dy, z += dz + (y > nyi ? 1 : 0), y -= (y > nyi ? nyi : 0)) {
        for (int x = 1 + threadIdx.x; x <= nxi; x += blockDim.x) {
            const long long I = lin(g, x, y, z);
            double fo = 0.0, mt = 0.0;
            for (int i = 0; i < g.D; ++i) {
                const double lo = u[I + i * g.N], hi = u[I + g.s[i] + i * g.N];
                fo += dmax(0.0, hi) + dmax(0.0, dneg(lo));   // WaterLily flux_out
                mt += dmax(dabs(lo), dabs(hi));              // maxTotalFlux
            }
            const unsigned long long b1 = nonneg_bits(fo), b2 = nonneg_bits(mt);
            a1 = b1 > a1 ? b1 : a1;
            a2 = b2 > a2 ? b2 : a2;
        }
    }
    a1 = warp_umax(a1);
    a2 = warp_umax(a2);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) {
        s1[w] = a1;
        s2[w] = a2;
    }
    __syncthreads();
    if (w == 0) {
        const int nw = blockDim.x >> 5;
        a1 = warp_umax(lane < nw ? s1[lane] : 0ull);
        a2 = warp_umax(lane < nw ? s2[lane] : 0ull);
        if (lane == 0) {
            atomicMax(out, a1);
            atomicMax(out + 1, a2);
        }
    }
}

}  // namespace

cudaError_t k_ustar(const MomConsts& k, const double* rhou, const double* f, double* ustar, cudaStream_t s) {
    { ustar_kern<<<ggrd(k.g), blk(), 0, s>>>(k, rhou, f, ustar); ia::note_launch(); }
    return cudaGetLastError();
}
cudaError_t k_stage_start(const MomConsts& k, const double* us, double* ud, const double* fs, double* fd, double* rhou,
                          cudaStream_t s) {
    if (k.g.D == 3) { stage_start_kern<3><<<ggrd(k.g), blk(), 0, s>>>(k, us, ud, fs, fd, rhou); ia::note_launch(); }
    else { stage_start_kern<2><<<ggrd(k.g), blk(), 0, s>>>(k, us, ud, fs, fd, rhou); ia::note_launch(); }
    return cudaGetLastError();
}
cudaError_t k_u2rhou(const MomConsts& k, double* rhou, const double* u, const double* f, cudaStream_t s) {
    { u2rhou_kern<<<igrd(k.g), blk(), 0, s>>>(k, rhou, u, f); ia::note_launch(); }
    return cudaGetLastError();
}
cudaError_t k_bc_vel(const MomConsts& k, double* a, const double* A, cudaStream_t s) {
    { bcvel_kern<<<unsigned((bc_plane_cells(k.g) + 255) / 256), 256, 0, s>>>(k, a, A[0], A[1], A[2]); ia::note_launch(); }
    return cudaGetLastError();
}
cudaError_t k_momflux(const MomConsts& k, int j, int limiter, const double* ustar, const double* rhouf_j,
                      const double* fold, double dt, double* Phi, cudaStream_t s) {
    FluxCtx F;
    F.k = k;
    F.j = j;
    F.lim = limiter;
    F.us = ustar;
    F.rj = rhouf_j;
    F.fold = fold;
    F.dt = dt;
    F.inv_dt = 1.0 / dt;
    F.half_inv_dt = 0.5 / dt;
    F.thr_l = k.lrho / dt;
    F.thr_1 = k.rho1 / dt;
    F.kl_l = dt * k.inv_lrho;
    F.kl_1 = dt * k.inv_rho1;
    switch (limiter) {
        case IA_LIMITER_UPWIND: { momflux_kern<IA_LIMITER_UPWIND><<<split_grid(k.g), blk(), 0, s>>>(F, Phi); ia::note_launch(); } break;
        case IA_LIMITER_MINMOD: { momflux_kern<IA_LIMITER_MINMOD><<<split_grid(k.g), blk(), 0, s>>>(F, Phi); ia::note_launch(); } break;
        case IA_LIMITER_VANALBADA1: { momflux_kern<IA_LIMITER_VANALBADA1><<<split_grid(k.g), blk(), 0, s>>>(F, Phi); ia::note_launch(); } break;
        case IA_LIMITER_SWEBY: { momflux_kern<IA_LIMITER_SWEBY><<<split_grid(k.g), blk(), 0, s>>>(F, Phi); ia::note_launch(); } break;
        case IA_LIMITER_SUPERBEE: { momflux_kern<IA_LIMITER_SUPERBEE><<<split_grid(k.g), blk(), 0, s>>>(F, Phi); ia::note_launch(); } break;
        case IA_LIMITER_TVDCEN: { momflux_kern<IA_LIMITER_TVDCEN><<<split_grid(k.g), blk(), 0, s>>>(F, Phi); ia::note_launch(); } break;
        case IA_LIMITER_TVDDOWN: { momflux_kern<IA_LIMITER_TVDDOWN><<<split_grid(k.g), blk(), 0, s>>>(F, Phi); ia::note_launch(); } break;
        default: { momflux_kern<IA_LIMITER_KOREN><<<split_grid(k.g), blk(), 0, s>>>(F, Phi); ia::note_launch(); } break;
    }
    return cudaGetLastError();
}
cudaError_t k_momupdate(const MomConsts& k, int j, const double* Phi, const double* uOld, const double* u1,
                        const double* u2, const int8_t* cbar, double dt, double* rhou, cudaStream_t s) {
    const Grid& g = k.g;
    const dim3 tg((g.n[0] - 2 + 31) / 32, (g.n[1] - 2 + 7) / 8, g.D == 3 ? (g.n[2] - 2 + MU_ZC - 1) / MU_ZC : 1);
    if (g.D == 3) { momupdate_kern<3><<<tg, blk(), 0, s>>>(k, j, Phi, uOld, u1 + j * g.N, u2 + j * g.N, cbar, dt, rhou); ia::note_launch(); }
    else { momupdate_kern<2><<<tg, blk(), 0, s>>>(k, j, Phi, uOld, u1 + j * g.N, u2 + j * g.N, cbar, dt, rhou); ia::note_launch(); }
    return cudaGetLastError();
}
cudaError_t k_visc(const MomConsts& k, const double* u, const double* f, double lmu, double mu, double* Phi6,
                   double* r, cudaStream_t s) {
    ViscCtx V;
    V.k = k;
    V.u = u;
    V.f = f;
    V.lmu = lmu;
    V.mu = mu;
    V.ratio = lmu / k.lrho;
    // getμ at faces with all four fractions 0 or all 1
    auto lin_prop = [](double s, double l) { return l + (1.0 - l) * s; };
    auto mu_at = [&](double s) {
        const double fac = (s > 0.5) ? 1.0 : lmu / k.lrho;
        const double a = lin_prop(s, lmu), b = fac * lin_prop(s, k.lrho);
        return mu * (b < a ? b : a);
    };
    V.mu_face0 = mu_at(0.0);
    V.mu_face1 = mu_at(1.0);
    if (k.g.D == 3) { viscflux_kern<3><<<split_grid(k.g), blk(), 0, s>>>(V, Phi6); ia::note_launch(); }
    else { viscflux_kern<2><<<split_grid(k.g), blk(), 0, s>>>(V, Phi6); ia::note_launch(); }
    { viscacc_kern<<<igrd(k.g), blk(), 0, s>>>(k.g, Phi6, r); ia::note_launch(); }
    return cudaGetLastError();
}
cudaError_t k_zero(double* a, long long n, cudaStream_t s) {
    { zero_kern<<<1216, 256, 0, s>>>(a, n); ia::note_launch(); }
    return cudaGetLastError();
}
cudaError_t k_surften(const MomConsts& k, const double* f, const double* prev0, double eta, double* fb, double* r,
                      int* list, unsigned int* count, cudaStream_t s) {
    const Grid& g = k.g;
    cudaMemsetAsync(count, 0, sizeof(unsigned int) * g.D, s);
    if (k.g.D == 3) { fbuffer_kern<3><<<ggrd(g), blk(), 0, s>>>(k, f, prev0, fb, list, count); ia::note_launch(); }
    else { fbuffer_kern<2><<<ggrd(g), blk(), 0, s>>>(k, f, prev0, fb, list, count); ia::note_launch(); }
    for (int d = 0; d < g.D; ++d) {
        double* fbd = fb + d * g.N;
        const int* ld = list + d * g.N;
        if (g.D == 2) { surften_kern<2><<<608, 64, 0, s>>>(k, d, f, fbd, eta, r, ld, count + d); ia::note_launch(); }
        else { surften_kern<3><<<608, 64, 0, s>>>(k, d, f, fbd, eta, r, ld, count + d); ia::note_launch(); }
    }
    return cudaGetLastError();
}
cudaError_t k_updateu(const MomConsts& k, double* u, double* rhou, const double* u0, const double* F, double dt,
                      const double* fref, const double* fupd, double w, bool write_rhou, cudaStream_t s) {
    const double a = 1.0 / w - 1.0;
    if (a == 0.0) { updateu_kern<true><<<igrd(k.g), blk(), 0, s>>>(k, u, rhou, u0, F, dt, fref, fupd, w, a, write_rhou); ia::note_launch(); }
    else { updateu_kern<false><<<igrd(k.g), blk(), 0, s>>>(k, u, rhou, u0, F, dt, fref, fupd, w, a, write_rhou); ia::note_launch(); }
    return cudaGetLastError();
}
cudaError_t k_updatel(const MomConsts& k, double* mu0, const double* f, cudaStream_t s) {
    if (k.g.D == 3) { updatel_kern<3><<<ggrd(k.g), blk(), 0, s>>>(k, mu0, f); ia::note_launch(); }
    else { updatel_kern<2><<<ggrd(k.g), blk(), 0, s>>>(k, mu0, f); ia::note_launch(); }
    return cudaGetLastError();
}
cudaError_t k_div_scale(const MomConsts& k, const double* u, double* zz, double* xx, double dt, cudaStream_t s) {
    { div_scale_kern<<<ggrd(k.g), blk(), 0, s>>>(k.g, u, zz, xx, dt); ia::note_launch(); }
    return cudaGetLastError();
}
cudaError_t k_correct(const MomConsts& k, double* u, const double* L, double* xx, double dt, cudaStream_t s) {
    if (k.g.D == 3) { correct_kern<3><<<igrd(k.g), blk(), 0, s>>>(k.g, u, L, xx); ia::note_launch(); }
    else { correct_kern<2><<<igrd(k.g), blk(), 0, s>>>(k.g, u, L, xx); ia::note_launch(); }
    { scale_kern<<<1216, 256, 0, s>>>(xx, k.g.N, 1.0 / dt); ia::note_launch(); }
    return cudaGetLastError();
}
cudaError_t k_cfl(const MomConsts& k, const double* u, unsigned long long* out2, cudaStream_t s) {
    const long long rows = (long long)(k.g.n[1] - 2) * (k.g.D == 3 ? k.g.n[2] - 2 : 1);
    { cfl_kern<<<int(rows < 1216 ? rows : 1216), 256, 0, s>>>(k.g, u, out2); ia::note_launch(); }
    return cudaGetLastError();
}
cudaError_t k_scale(double* a, long long n, double f, cudaStream_t s) {
    { scale_kern<<<1216, 256, 0, s>>>(a, n, f); ia::note_launch(); }
    return cudaGetLastError();
}
cudaError_t k_average(double* a, const double* b, long long n, cudaStream_t s) {
    { average_kern<<<1216, 256, 0, s>>>(a, b, n); ia::note_launch(); }
    return cudaGetLastError();
}

}  // namespace ia
