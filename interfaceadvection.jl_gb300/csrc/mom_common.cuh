// Launch shapes, context structs and the rare-path FP64 helpers shared by the FP64 momentum kernels
// (mom.cu) and their float-float counterparts (mom_ff.cu).  Everything here has internal linkage:
// each translation unit that includes it gets its own copy.
#pragma once
#include <cuda_runtime.h>

#include "ia_bc.cuh"
#include "ia_core.cuh"
#include "mom.cuh"

namespace ia {
namespace {

inline dim3 blk() { return dim3(32, 8, 1); }

// Interior-cell launch: lane 0 of the first block sits on cell 1, so a row of 32k interior
// cells fills k warps exactly and no warp spends FP64 issue slots on a ghost-cell lane.
inline dim3 igrd(const Grid& g) {
    return dim3((g.n[0] - 2 + 31) / 32, (g.n[1] - 2 + 7) / 8, g.D == 3 ? g.n[2] - 2 : 1);
}
#define ICELL_XYZ                                                                     \
    const int x = 1 + blockIdx.x * blockDim.x + threadIdx.x;                          \
    const int y = 1 + blockIdx.y * blockDim.y + threadIdx.y;                          \
    const int z = g.D == 3 ? 1 + int(blockIdx.z) : 0;                                 \
    if (x > g.n[0] - 2 || y > g.n[1] - 2) return;

// Whole-grid launch: the x-range [1, n-2] one cell per lane, then one more block column whose
// first warp takes the ghost cells x = 0 and x = n-1 of the block's 8 rows, so that a row of
// 32k interior cells fills k warps and no warp of FP64 work runs with two lanes.
inline dim3 ggrd(const Grid& g) { return dim3((g.n[0] - 2 + 31) / 32 + 1, (g.n[1] + 7) / 8, g.n[2]); }
#define GCELL_XYZ                                                                     \
    int x, y;                                                                         \
    const int z = blockIdx.z;                                                         \
    if (blockIdx.x + 1 < gridDim.x) {                                                 \
        x = 1 + int(blockIdx.x) * 32 + int(threadIdx.x);                              \
        y = int(blockIdx.y) * 8 + int(threadIdx.y);                                   \
        if (x > g.n[0] - 2) return;                                                   \
    } else {                                                                          \
        if (threadIdx.y != 0 || threadIdx.x >= 16) return;                            \
        x = (threadIdx.x & 1) ? g.n[0] - 1 : 0;                                       \
        y = int(blockIdx.y) * 8 + (int(threadIdx.x) >> 1);                            \
    }                                                                                 \
    if (y >= g.n[1]) return;

// Face-flux launch (momentum flux, viscous flux): the x-range [3, n-3], whose faces and
// edges need no boundary rule, one cell per lane; then one more block column whose first
// warp takes the x-boundary cells {1, 2, n-2, n-1} of the block's 8 rows.  A warp then runs
// either the bulk path or the boundary path for all its lanes: FP64 issues per warp
// instruction, whatever the number of active lanes, so a warp that mixes the two pays for both.
inline dim3 split_grid(const Grid& g) {
    const int wi = g.n[0] > 5 ? (g.n[0] - 5 + 31) / 32 : 0;
    return dim3(wi + 1, (g.n[1] + 7) / 8, g.n[2]);
}
#define SPLIT_XYZ                                                                     \
    int x, y;                                                                         \
    const int z = blockIdx.z;                                                         \
    if (blockIdx.x + 1 < gridDim.x) {                                                 \
        x = 3 + int(blockIdx.x) * 32 + int(threadIdx.x);                              \
        y = int(blockIdx.y) * 8 + int(threadIdx.y);                                   \
        if (x > g.n[0] - 3) return;                                                   \
    } else {                                                                          \
        if (threadIdx.y != 0) return;                                                 \
        const int kb = int(threadIdx.x) & 3;                                          \
        x = kb < 2 ? 1 + kb : g.n[0] - 4 + kb;                                        \
        if (kb >= 2 && x <= 2) return;                                                \
        y = int(blockIdx.y) * 8 + (int(threadIdx.x) >> 2);                            \
    }                                                                                 \
    if (y >= g.n[1]) return;

// x / getρ and x · getρ for a face between cells with fractions fa, fb (src/VOFutil.jl:176,
// 198-201).  The mixed-face forms stay out of line: inlined, they are if-converted and their
// predicated-off FP64 instructions would take FP64 issue slots on every bulk face.
__device__ __noinline__ double div_rho_mixed(double lrho, double one_m, double v, double fa, double fb) {
    return v / (lrho + one_m * ((fa + fb) / 2.0));
}
__device__ __noinline__ double mul_rho_mixed(double lrho, double one_m, double v, double fa, double fb) {
    return v * (lrho + one_m * ((fa + fb) / 2.0));
}
__device__ __forceinline__ double div_rho(const MomConsts& k, double v, double fa, double fb) {
    const unsigned long long a = dbits(fa), b = dbits(fb);
    if (a == b && a == 0ull) return v * k.inv_lrho;
    if (a == b && a == kOneBits) return v * k.inv_rho1;
    return div_rho_mixed(k.lrho, k.one_m, v, fa, fb);
}
__device__ __forceinline__ double mul_rho(const MomConsts& k, double v, double fa, double fb) {
    const unsigned long long a = dbits(fa), b = dbits(fb);
    if (a == b && a == 0ull) return v * k.lrho;
    if (a == b && a == kOneBits) return v * k.rho1;
    return mul_rho_mixed(k.lrho, k.one_m, v, fa, fb);
}

struct FluxCtx {
    MomConsts k;
    int j, lim;
    const double* us;
    const double* rj;     // ρuf[:, j] before the 1/δt scaling
    const double* fold;
    double dt, inv_dt, half_inv_dt;
    // pure-phase faces: m_old < m_out  <=>  |Ψ| > thr (thr = m_old/δt), l₂ = |Ψ|·kl (kl = δt/m_old)
    double thr_l, thr_1, kl_l, kl_1;
};

// ρuf[X, j] (raw, before 1/δt) or, on a BC! face, the boundary velocity (returns true)
__device__ __forceinline__ bool rraw(const FluxCtx& F, int c[3], double& v) {
    const Grid& g = F.k.g;
    if (vel_bc(g, F.j, c)) {
        v = F.k.uBC[F.j];
        return true;
    }
    v = F.rj[lin3(g, c)];
    return false;
}
// m_old = λρ + (1-λρ) dρ[X, i] with dρ = BCv!(f2face!(f_old)): kind 1 light, 2 dark (constants),
// 0 mixed (value in m).  The upper normal face of a zero-gradient dimension is never written by
// the reference and keeps the 1 it is initialised with (src/cVOF.jl:74).
__device__ __forceinline__ int m_old_kind(const FluxCtx& F, int i, int c[3], double& m) {
    const Grid& g = F.k.g;
    if (face_bc(g, i, c)) return 2;
    const long long P = lin3(g, c);
    const double fa = F.fold[P], fb = F.fold[P - g.s[i]];
    const unsigned long long a = dbits(fa), b = dbits(fb);
    if (a == b && a == 0ull) return 1;
    if (a == b && a == kOneBits) return 2;
    m = F.k.lrho + F.k.one_m * ((fa + fb) / 2.0);
    return 0;
}

// l₂ = m_out / m_old on a face whose old fractions fa, fb are not both 0 or both 1, or -1 when
// m_old < m_out (the flux is then Ψ v_I).  Out of line so that bulk faces do not issue it.
__device__ __noinline__ double l2_mixed(const FluxCtx& F, double fa, double fb, double aP) {
    const double mOld = F.k.lrho + F.k.one_m * ((fa + fb) / 2.0);
    const double mOut = aP * F.dt;
    if (dlt(mOld, mOut)) return -1.0;
    return mOut / mOld;
}

constexpr int MU_ZC = 16;


struct ViscCtx {
    MomConsts k;
    const double* u;
    const double* f;
    double lmu, mu, mu_face0, mu_face1;   // μ at full-light / full-dark faces
    double ratio;                         // λμ/λρ
};

// fFace = BCv!(f2face!(f)); the reference's fFace buffer aliases n̂, whose upper
// normal face still holds uStar's Dirichlet value u_BC[d] from the last momentum sweep.
__device__ __forceinline__ double fface(const ViscCtx& V, int d, int c[3]) {
    const Grid& g = V.k.g;
    if (face_bc(g, d, c)) return V.k.uBC[d];
    const long long P = lin3(g, c);
    const double fa = V.f[P], fb = V.f[P - g.s[d]];
    if (dbits(fa) == dbits(fb)) return fa;
    return (fa + fb) / 2.0;
}

// getμ(i,j,I,fFace,λμ,μ,λρ) (src/VOFutil.jl:186-191).  Kept out of line: inlined, its
// mixed-face arithmetic is if-converted and the predicated-off FP64 instructions still take
// FP64 issue slots in every bulk cell.
__device__ __noinline__ double get_mu(const ViscCtx& V, int i, int j, const int cI[3]) {
    int a[3] = {cI[0], cI[1], cI[2]}, b[3] = {cI[0], cI[1], cI[2]}, c[3] = {cI[0], cI[1], cI[2]},
        d[3] = {cI[0], cI[1], cI[2]};
    a[j] -= 1;
    c[i] -= 1;
    const double f1 = fface(V, i, a), f2 = fface(V, i, b), f3 = fface(V, j, c), f4 = fface(V, j, d);
    const unsigned long long b1 = dbits(f1);
    if (b1 == dbits(f2) && b1 == dbits(f3) && b1 == dbits(f4)) {
        if (b1 == 0ull) return V.mu_face0;
        if (b1 == kOneBits) return V.mu_face1;
    }
    const double s = (f1 + f2 + f3 + f4) / 4.0;
    const double fr = V.k.lrho < 1.0 ? dmin(dmin(f1, f2), dmin(f3, f4)) : dmax(dmax(f1, f2), dmax(f3, f4));
    const double fac = dlt(0.5, s) ? 1.0 : V.ratio;
    return V.mu * dmin(V.lmu + (1.0 - V.lmu) * s, fac * (V.k.lrho + V.k.one_m * fr));
}

// getμ for an edge/face whose cells all lie at least two cells inside the grid (no ghost or
// boundary-face rule applies): the fractions of the 3 (i == j) or 4 cells decide a pure phase
// with integer compares; anything else goes to the general helper.
__device__ __forceinline__ double get_mu_inner(const ViscCtx& V, int i, int j, const int c[3], long long K) {
    const Grid& g = V.k.g;
    const double* f = V.f;
    const unsigned long long a = dbits(f[K]), b = dbits(f[K - g.s[i]]);
    const unsigned long long e = dbits(i == j ? f[K - 2 * g.s[i]] : f[K - g.s[j]]);
    const unsigned long long d = i == j ? a : dbits(f[K - g.s[i] - g.s[j]]);
    if (a == b && a == e && a == d) {
        if (a == 0ull) return V.mu_face0;
        if (a == kOneBits) return V.mu_face1;
    }
    return get_mu(V, i, j, c);
}

__device__ __forceinline__ int pair_index(int D, int i, int j) {
    if (i == j) return i;
    const int a = i < j ? i : j, b = i < j ? j : i;
    return D + (a == 0 ? (b - 1) : 2);   // (0,1)->D, (0,2)->D+1, (1,2)->D+2
}

}  // namespace
}  // namespace ia
