// Variable-coefficient pressure Poisson solve of the projection step
// (InterfaceAdvection.jl src/flow.jl:328-347, where WaterLily's
// MultiLevelPoisson `solver!` runs V-cycles inside a PCG wrapper).
//
// Operator (WaterLily `mult`): (A x)_I = Σ_i L[I,i] x[I-δi] + L[I+δi,i] x[I+δi]
// + D_I x_I with D_I = -Σ_i (L[I,i] + L[I+δi,i]); L = μ₀ = 1/ρ on faces, zero
// on wall faces, periodic dimensions wrap.  The solver is this library's own:
//
//  * geometric multigrid on cell-centred levels (2x coarsening while every
//    interior extent is even and >= 4); coarse face coefficient = ½ Σ of the
//    2^(D-1) fine faces it covers; restriction sums the 2^D children,
//    prolongation injects; red-black Gauss-Seidel, ν₁ sweeps red→black
//    before and ν₂ black→red after, so the V-cycle is a symmetric
//    preconditioner; the coarsest level is solved by one block with a fixed
//    number of symmetric sweeps on the mean-free right-hand side;
//  * flexible CG in FP64 around it (β from the residual change, so an
//    inexact FP32 V-cycle stays admissible), stopping on the L∞ norm of the
//    FP64 true residual of the dt-scaled system.
//
// IA_POISSON_FP64 runs the V-cycle in FP64; IA_POISSON_MIXED runs it in FP32
// (FP32 copies of every level's operator), the defect correction, matvec,
// dot products and updates staying FP64.  IA_POISSON_LEARNED keeps the MIXED
// structure and preconditions the inner FCG with the conv net (nn.cu), composed
// with the V-cycle (hybrid) or alone; an outer correction that fails to halve
// the FP64 true residual switches the rest of the solve to the plain V-cycle.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "capi_internal.cuh"
#include "ia_bc.cuh"
#include "ff.cuh"
#include "poisson.cuh"

namespace ia {

namespace {

inline dim3 blk() { return dim3(32, 8, 1); }
inline dim3 grd(const Grid& g) { return dim3((g.n[0] + 31) / 32, (g.n[1] + 7) / 8, g.n[2]); }

// neighbour offset of interior cell coordinate ci along dimension i (periodic wrap;
// on a wall the ghost is read but its face coefficient is zero)
__device__ __forceinline__ long long lo_off(const Grid& g, int i, int ci) {
    return (g.isper(i) && ci == 1) ? (long long)(g.n[i] - 3) * g.s[i] : -g.s[i];
}
__device__ __forceinline__ long long hi_off(const Grid& g, int i, int ci) {
    return (g.isper(i) && ci == g.n[i] - 2) ? -(long long)(g.n[i] - 3) * g.s[i] : g.s[i];
}

template <class T>
__device__ __forceinline__ T offdiag(const Grid& g, const T* L, const T* x, long long I, const int c[3]) {
    T a = T(0);
    for (int i = 0; i < g.D; ++i)
        a += L[I + i * g.N] * x[I + lo_off(g, i, c[i])] + L[I + g.s[i] + i * g.N] * x[I + hi_off(g, i, c[i])];
    return a;
}

// face coefficient as the arithmetic type of the sweep (the finest mixed level may store them as FP16)
__device__ __forceinline__ float cf(float v) { return v; }
__device__ __forceinline__ double cf(double v) { return v; }
__device__ __forceinline__ float cf(__half v) { return __half2float(v); }

// ---- dimension-specialised stencil with 32-bit cell offsets (a grid holds < 2^31 cells)
struct Nb {
    int xl, xh, yl, yh, zl, zh;   // offsets of the six neighbours; periodic ends wrap
};
template <int D>
__device__ __forceinline__ Nb nb_of(const Grid& g, int x, int y, int z) {
    Nb o;
    const int s1 = int(g.s[1]), s2 = int(g.s[2]);
    o.xl = (g.isper(0) && x == 1) ? g.n[0] - 3 : -1;
    o.xh = (g.isper(0) && x == g.n[0] - 2) ? 3 - g.n[0] : 1;
    o.yl = (g.isper(1) && y == 1) ? (g.n[1] - 3) * s1 : -s1;
    o.yh = (g.isper(1) && y == g.n[1] - 2) ? (3 - g.n[1]) * s1 : s1;
    o.zl = o.zh = 0;
    if (D == 3) {
        o.zl = (g.isper(2) && z == 1) ? (g.n[2] - 3) * s2 : -s2;
        o.zh = (g.isper(2) && z == g.n[2] - 2) ? (3 - g.n[2]) * s2 : s2;
    }
    return o;
}
// Σ_i L[I,i] v[I-δi] + L[I+δi,i] v[I+δi]  (same order as offdiag)
template <int D, class T, class TL>
__device__ __forceinline__ T off7(const Grid& g, const TL* __restrict__ L, const T* v, int I, const Nb& o) {
    const int s1 = int(g.s[1]), s2 = int(g.s[2]);
    const TL* L1 = L + g.N;
    T a = cf(L[I]) * v[I + o.xl] + cf(L[I + 1]) * v[I + o.xh];
    a += cf(L1[I]) * v[I + o.yl] + cf(L1[I + s1]) * v[I + o.yh];
    if (D == 3) {
        const TL* L2 = L1 + g.N;
        a += cf(L2[I]) * v[I + o.zl] + cf(L2[I + s2]) * v[I + o.zh];
    }
    return a;
}
// D_I = -Σ_i (L[I,i] + L[I+δi,i])
template <int D, class TL>
__device__ __forceinline__ auto diag7(const Grid& g, const TL* __restrict__ L, int I) -> decltype(cf(L[0])) {
    using T = decltype(cf(L[0]));
    const int s1 = int(g.s[1]), s2 = int(g.s[2]);
    const TL* L1 = L + g.N;
    T dd = T(0);
    dd -= cf(L[I]) + cf(L[I + 1]);
    dd -= cf(L1[I]) + cf(L1[I + s1]);
    if (D == 3) {
        const TL* L2 = L1 + g.N;
        dd -= cf(L2[I]) + cf(L2[I + s2]);
    }
    return dd;
}
// interior-cell launch: x, y from the 2D block, z from blockIdx.z (3D) or 0 (2D)
#define CELL_INTERIOR(g)                                                  \
    const int x = 1 + blockIdx.x * blockDim.x + threadIdx.x;              \
    const int y = 1 + blockIdx.y * blockDim.y + threadIdx.y;              \
    const int z = D == 3 ? 1 + int(blockIdx.z) : 0;                       \
    if (x > (g).n[0] - 2 || y > (g).n[1] - 2) return;                     \
    const int I = x + y * int((g).s[1]) + z * int((g).s[2]);
inline dim3 cell_grid(const Grid& g) {
    return dim3((g.n[0] - 2 + 31) / 32, (g.n[1] - 2 + 7) / 8, g.D == 3 ? g.n[2] - 2 : 1);
}
// launch K<D> for the grid's dimension
#define LAUNCH_D(gg, K, grid, block, ...)                                             \
    do {                                                                              \
        if ((gg).D == 3) { K<3><<<grid, block, 0, st>>>(__VA_ARGS__); ia::note_launch(); } \
        else { K<2><<<grid, block, 0, st>>>(__VA_ARGS__); ia::note_launch(); }             \
    } while (0)

#define INTERIOR_XYZ                                                                                     \
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;     \
    const int z = blockIdx.z;                                                                            \
    if (x < 1 || y < 1 || x > g.n[0] - 2 || y > g.n[1] - 2) return;                                      \
    if (g.D == 3 && (z < 1 || z > g.n[2] - 2)) return;                                                   \
    [[maybe_unused]] const int c[3] = {x, y, z};                                                         \
    const long long I = lin(g, x, y, z);

template <class T>
__global__ void set_diag_k(Grid g, const T* __restrict__ L, T* __restrict__ iD) {
    INTERIOR_XYZ
    T dd = T(0);
    for (int i = 0; i < g.D; ++i) dd -= L[I + i * g.N] + L[I + g.s[i] + i * g.N];
    const T eps = sizeof(T) == 8 ? T(2.220446049250313e-16) : T(1.1920929e-7);
    iD[I] = (dd * dd < T(2) * eps) ? T(0) : T(1) / dd;
}

// Coarse face coefficients: ½ Σ over the fine faces covering each coarse face
// (all coarse faces 1..n-1 along i, interior elsewhere).
template <class T>
__global__ void restrict_L_k(Grid gc, Grid gf, const T* __restrict__ Lf, T* __restrict__ Lc) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z;
    if (x >= gc.n[0] || y >= gc.n[1]) return;
    const int c[3] = {x, y, z};
    const long long Ic = lin(gc, x, y, z);
    for (int i = 0; i < gc.D; ++i) {
        bool ok = true;
        for (int e = 0; e < gc.D; ++e) {
            const int hi = (e == i) ? gc.n[e] - 1 : gc.n[e] - 2;
            if (c[e] < 1 || c[e] > hi) ok = false;
        }
        if (!ok) continue;
        // fine base cell of the face: coordinate 2c-1 in every dimension
        int fb[3] = {2 * c[0] - 1, 2 * c[1] - 1, gc.D == 3 ? 2 * c[2] - 1 : 0};
        T s = T(0);
        const int o1 = (i == 0) ? 1 : 0, o2 = (i == 2) ? 1 : 2;   // the other dimensions
        const int n1 = 2, n2 = (gc.D == 3) ? 2 : 1;
        for (int b = 0; b < n2; ++b)
            for (int a = 0; a < n1; ++a) {
                int q[3] = {fb[0], fb[1], fb[2]};
                q[o1] += a;
                if (gc.D == 3) q[o2] += b;
                s += Lf[lin(gf, q[0], q[1], q[2]) + i * gf.N];
            }
        Lc[Ic + i * gc.N] = T(0.5) * s;
    }
}

// Red-black Gauss-Seidel half-sweep, one thread per cell of the colour: thread tx takes the pair of
// interior cells (1 + 2tx, 2 + 2tx) of its row and updates the one of this colour, so no
// lane idles; the diagonal comes from the face coefficients the update reads anyway
// (same value and zero-diagonal rule as set_diag_k).
// With PROL (over-relaxed first red half-sweep of a post-smoothing whose prolongation is fused
// into the sweeps) the cell's previous value is x + the injected coarse correction.
// In 3D a thread takes its pair in RB_ZT consecutive z planes and reads every plane's operands before
// it stores: a half-sweep reads only the other colour, so no plane's store changes what another plane
// reads, and the loads of all planes are in flight at once (the z neighbours of one plane are the x
// neighbours of the next, a repeated address).  The values are those of one plane per thread.
constexpr int RB_ZT = 2;
inline dim3 pair_grid(const Grid& g) {
    const int pairs = (g.n[0] - 2 + 1) / 2;
    return dim3((pairs + 31) / 32, (g.n[1] - 2 + 7) / 8, g.D == 3 ? g.n[2] - 2 : 1);
}
inline dim3 pair_tile_grid(const Grid& g) {
    const int pairs = (g.n[0] - 2 + 1) / 2;
    return dim3((pairs + 31) / 32, (g.n[1] - 2 + 7) / 8, g.D == 3 ? (g.n[2] - 2 + RB_ZT - 1) / RB_ZT : 1);
}
template <class T, int D, bool PROL = false, class TL = T>
__global__ void rbgs_pair_k(Grid g, int y0, int y1, const TL* __restrict__ L, const T* __restrict__ b,
                            T* __restrict__ xv, int color, T omega, Grid gc = Grid(),
                            const T* __restrict__ xc = nullptr) {
    const int y = y0 + int(blockIdx.y * blockDim.y + threadIdx.y);   // rows [y0, y1) of the interior
    if (y >= y1) return;
    const int xp = 1 + 2 * (blockIdx.x * blockDim.x + threadIdx.x);
    const int z0 = D == 3 ? 1 + RB_ZT * int(blockIdx.z) : 0;
    const T eps = sizeof(T) == 8 ? T(2.220446049250313e-16) : T(1.1920929e-7);
    // plane k's cell of this colour and its operands: the off-diagonal sum, the diagonal, b and
    // (over-relaxed) the previous value
    auto cell_of = [&](int z) {
        int x = xp;
        if (((x + y + z) & 1) != color) ++x;
        return x;
    };
    auto load = [&](int x, int z, int& I, T& off, T& dd, T& bv, T& xo) {
        I = x + y * int(g.s[1]) + z * int(g.s[2]);
        const Nb o = nb_of<D>(g, x, y, z);
        off = off7<D>(g, L, xv, I, o);
        dd = diag7<D>(g, L, I);
        bv = b[I];
        if (omega != T(1)) {
            xo = xv[I];
            if (PROL) xo += xc[lin(gc, (x + 1) / 2, (y + 1) / 2, D == 3 ? (z + 1) / 2 : 0)];
        }
    };
    auto store = [&](int I, T off, T dd, T bv, T xo) {
        const T iD = (dd * dd < T(2) * eps) ? T(0) : T(1) / dd;
        const T gs = (bv - off) * iD;
        if (omega == T(1)) xv[I] = gs;
        else xv[I] = xo + omega * (gs - xo);   // over-relaxation: x + ω (x_GS - x)
    };
    const int xmax = g.n[0] - 2;
    if (D == 3 && z0 + RB_ZT - 1 <= g.n[2] - 2) {
        int I[RB_ZT];
        T off[RB_ZT], dd[RB_ZT], bv[RB_ZT], xo[RB_ZT];
        bool ok[RB_ZT];
#pragma unroll
        for (int k = 0; k < RB_ZT; ++k) {
            const int x = cell_of(z0 + k);
            ok[k] = x <= xmax;
            xo[k] = T(0);
            if (ok[k]) load(x, z0 + k, I[k], off[k], dd[k], bv[k], xo[k]);
        }
#pragma unroll
        for (int k = 0; k < RB_ZT; ++k)
            if (ok[k]) store(I[k], off[k], dd[k], bv[k], xo[k]);
        return;
    }
    for (int k = 0; k < (D == 3 ? RB_ZT : 1); ++k) {
        const int z = z0 + k;
        if (D == 3 && z > g.n[2] - 2) break;
        const int x = cell_of(z);
        if (x > xmax) continue;
        int I;
        T off, dd, bv, xo = T(0);
        load(x, z, I, off, dd, bv, xo);
        store(I, off, dd, bv, xo);
    }
}

// ---- first half-sweep of a smoothing, fused with the pass before it.  A red update reads only
// black neighbours, so the red values that precede a smoothing's first (black) half-sweep are
// consumed by that half-sweep alone: they are computed here where read, b (1/D) for the
// pre-smoothing from x = 0 (the first red sweep, whose neighbours are zero) and x + the
// injected coarse correction for the post-smoothing (prolong_k's values, interior cells only).  The red cells are written only for
// a pre-smoothing of one sweep (write_red), whose red values are part of its result.
template <class T, bool PROL>
__device__ __forceinline__ T first_nb(const Grid& g, const Grid& gc, const T* __restrict__ b,
                                      const T* __restrict__ iD, const T* __restrict__ xc, const T* xv, int J,
                                      int cx, int cy, int cz, T omega) {
    // J, (cx, cy, cz): index and (periodically wrapped) coordinates of the neighbour
    const bool in = cx >= 1 && cx <= g.n[0] - 2 && cy >= 1 && cy <= g.n[1] - 2 &&
                    (g.D == 2 || (cz >= 1 && cz <= g.n[2] - 2));
    if (!in) return xv[J];
    if (PROL) return xv[J] + xc[lin(gc, (cx + 1) / 2, (cy + 1) / 2, g.D == 3 ? (cz + 1) / 2 : 0)];
    return omega == T(1) ? b[J] * iD[J] : omega * (b[J] * iD[J]);
}

template <class T, int D, bool PROL, class TL = T>
__global__ void rbgs_first_k(Grid g, int y0, int y1, Grid gc, const TL* __restrict__ L, const T* __restrict__ b,
                             const T* __restrict__ iD, const T* __restrict__ xc, T* __restrict__ xv, int write_red,
                             T omega) {
    const int y = y0 + int(blockIdx.y * blockDim.y + threadIdx.y);   // rows [y0, y1) of the interior
    const int z = D == 3 ? 1 + int(blockIdx.z) : 0;
    if (y >= y1) return;
    const int x0 = 1 + 2 * (blockIdx.x * blockDim.x + threadIdx.x);
    const bool blk0 = ((x0 + y + z) & 1) == 1;
    const int x = blk0 ? x0 : x0 + 1, xr = blk0 ? x0 + 1 : x0;   // black and red cell of the pair
    const int s1 = int(g.s[1]), s2 = int(g.s[2]);
    if (!PROL && write_red && xr <= g.n[0] - 2) {
        const int Ir = xr + y * s1 + z * s2;
        xv[Ir] = omega == T(1) ? b[Ir] * iD[Ir] : omega * (b[Ir] * iD[Ir]);
    }
    if (x > g.n[0] - 2) return;
    const int I = x + y * s1 + z * s2;
    const TL* L1 = L + g.N;
    const TL* L2 = L1 + g.N;
    // the six neighbour values, then one shared accumulation (the same sums in the same order
    // whichever way the values were found)
    T v[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
    if (x >= 2 && x <= g.n[0] - 3 && y >= 2 && y <= g.n[1] - 3 && (D == 2 || (z >= 2 && z <= g.n[2] - 3))) {
        // every neighbour interior, no wrap: the coarse parent of the neighbour below (above) along
        // e is the cell's own parent, or the one below (above) when the coordinate is odd (even)
        const int J[6] = {I - 1, I + 1, I - s1, I + s1, I - s2, I + s2};
        if (PROL) {
            const int g1 = int(gc.s[1]), g2 = int(gc.s[2]);
            const int P = (x + 1) / 2 + ((y + 1) / 2) * g1 + (D == 3 ? ((z + 1) / 2) * g2 : 0);
            const int Pn[6] = {P - ((x & 1) ? 1 : 0), P + ((x & 1) ? 0 : 1), P - ((y & 1) ? g1 : 0),
                               P + ((y & 1) ? 0 : g1), P - ((z & 1) ? g2 : 0), P + ((z & 1) ? 0 : g2)};
#pragma unroll
            for (int q = 0; q < 2 * D; ++q) v[q] = xv[J[q]] + xc[Pn[q]];
        } else {
#pragma unroll
            for (int q = 0; q < 2 * D; ++q) v[q] = omega == T(1) ? b[J[q]] * iD[J[q]] : omega * (b[J[q]] * iD[J[q]]);
        }
    } else {
        const Nb o = nb_of<D>(g, x, y, z);
        const int xl = (g.isper(0) && x == 1) ? g.n[0] - 2 : x - 1, xh = (g.isper(0) && x == g.n[0] - 2) ? 1 : x + 1;
        const int yl = (g.isper(1) && y == 1) ? g.n[1] - 2 : y - 1, yh = (g.isper(1) && y == g.n[1] - 2) ? 1 : y + 1;
        v[0] = first_nb<T, PROL>(g, gc, b, iD, xc, xv, I + o.xl, xl, y, z, omega);
        v[1] = first_nb<T, PROL>(g, gc, b, iD, xc, xv, I + o.xh, xh, y, z, omega);
        v[2] = first_nb<T, PROL>(g, gc, b, iD, xc, xv, I + o.yl, x, yl, z, omega);
        v[3] = first_nb<T, PROL>(g, gc, b, iD, xc, xv, I + o.yh, x, yh, z, omega);
        if (D == 3) {
            const int zl = (g.isper(2) && z == 1) ? g.n[2] - 2 : z - 1, zh = (g.isper(2) && z == g.n[2] - 2) ? 1 : z + 1;
            v[4] = first_nb<T, PROL>(g, gc, b, iD, xc, xv, I + o.zl, x, y, zl, omega);
            v[5] = first_nb<T, PROL>(g, gc, b, iD, xc, xv, I + o.zh, x, y, zh, omega);
        }
    }
    T a = cf(L[I]) * v[0] + cf(L[I + 1]) * v[1];
    a += cf(L1[I]) * v[2] + cf(L1[I + s1]) * v[3];
    if (D == 3) a += cf(L2[I]) * v[4] + cf(L2[I + s2]) * v[5];
    const T dd = diag7<D>(g, L, I);
    const T eps = sizeof(T) == 8 ? T(2.220446049250313e-16) : T(1.1920929e-7);
    const T iDI = (dd * dd < T(2) * eps) ? T(0) : T(1) / dd;
    const T gs = (b[I] - a) * iDI;
    if (omega == T(1)) {
        xv[I] = gs;
    } else if (PROL) {   // over-relaxation from the prolongated value of this (black) cell
        const T xo = xv[I] + xc[lin(gc, (x + 1) / 2, (y + 1) / 2, D == 3 ? (z + 1) / 2 : 0)];
        xv[I] = xo + omega * (gs - xo);
    } else {             // from x = 0
        xv[I] = omega * gs;
    }
}

// ---- temporally blocked red-black Gauss-Seidel (3D, FP32): S half-sweeps in one launch.
// A block owns a TB_X x TB_Y column of interior cells and a range of z-planes and marches up
// z as a wavefront: at step t half-sweep s works on plane t - s over the column widened by
// S-1-s cells on every side, so that half-sweep s+1 finds every neighbour it reads in shared
// memory (three planes per half-sweep).  The widened parts are recomputed by every block that
// needs them, from the same inputs with the same arithmetic, so a cell has one value whichever
// block computes it; only its owner writes it.  Half-sweep s updates colour (c0 + s) & 1 with
// rbgs_pair_k's sums in rbgs_pair_k's order and the stored inverse diagonal (set_diag_k, the
// same formula).  A cell ends in x_out with the value of the last half-sweep of its colour.
// The input is zero (pre-smoothing: the V-cycle starts from x = 0) or x_in plus the injection
// prolongation of a coarse correction (post-smoothing).  Periodic dimensions wrap the widened
// column onto the grid (an even number of interior cells keeps the colouring); along a wall
// the cells outside the interior hold zero and their face coefficients are zero.
constexpr int TB_X = 32, TB_Y = 16, TB_T = 256;

struct TbArgs {
    Grid g, gc;            // level, coarse level (prolongation)
    const float* L;
    const float* b;
    const float* iD;
    const float* xin;      // post-smoothing input (null: start from zero)
    const float* xc;       // coarse correction added to xin (or null)
    float* xout;
    int c0;                // colour of the first half-sweep
    int zchunk;            // z-planes owned by a block
};

// grid coordinate of the logical coordinate l along e: periodic images wrap onto the
// interior, wall cells outside the interior are not valid
__device__ __forceinline__ int tb_wrap(const Grid& g, int e, int l, bool& ok) {
    const int m = g.n[e] - 2;
    if (g.isper(e)) {
        int p = l;
        while (p < 1) p += m;
        while (p > m) p -= m;
        ok = true;
        return p;
    }
    ok = l >= 1 && l <= m;
    return l;
}

__device__ __forceinline__ int tb_slot(int zl) { return (zl + 3 * 64) % 3; }

template <int S, bool ZERO>
__global__ void __launch_bounds__(TB_T, 4) rbgs_tb_k(TbArgs a) {
    // frame position (fx, fy) <-> logical cell (ox - S + fx, oy - S + fy).  A frame row is
    // stored as its even-fx half then its odd-fx half, so that the cells of one colour in a row
    // are contiguous.  Threads own pairs (2p, 2p+1) of a row: the frame starts on an odd logical
    // x and every level has an even number of interior cells per dimension, so the two cells of
    // a pair are both interior or both not, and a periodic wrap never falls between them.
    constexpr int FX = TB_X + 2 * S, FY = TB_Y + 2 * S, FN = FX * FY, HX = FX / 2;
    constexpr int RIN = ZERO ? 0 : 1;                 // ring 0 holds the input planes (post)
    constexpr int NIN = (FN + TB_T - 1) / TB_T;       // input cells per thread
    constexpr int F_VALID = 1, F_OWNED = 2, F_PAR = 4, F_LO = 8, F_HI = 16, F_USE = 32;
    __shared__ float ring[RIN + S - 1][3][FN];
    const Grid& g = a.g;
    const int tid = threadIdx.x;
    const int ox = 1 + int(blockIdx.x) * TB_X, oy = 1 + int(blockIdx.y) * TB_Y;
    const int nzi = g.n[2] - 2;
    const int z0 = 1 + int(blockIdx.z) * a.zchunk;
    if (z0 > nzi) return;
    const int z1 = min(z0 + a.zchunk, nzi + 1);
    const int s1 = int(g.s[1]), s2 = int(g.s[2]);
    const float* __restrict__ L0 = a.L;
    const float* __restrict__ L1 = a.L + g.N;
    const float* __restrict__ L2 = a.L + 2 * g.N;

    // pair slots of each half-sweep: frame index of the even cell, grid offset (x, y) of the
    // even cell, flags (valid, owned by this block, (x + y) parity, region edge pairs)
    int sq[S][2], sxy[S][2], sfl[S][2];
#pragma unroll
    for (int s = 0; s < S; ++s) {
        const int hs = S - 1 - s;
        const int plo = (S - hs) / 2, phi = (S + TB_X + hs + 1) / 2;
        const int np = phi - plo, rows = TB_Y + 2 * hs;
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const int it = tid + k * TB_T;
            sfl[s][k] = 0;
            sq[s][k] = 0;
            sxy[s][k] = 0;
            if (it >= np * rows) continue;
            const int r = it / np, p = plo + (it - r * np);
            const int fy = S - hs + r;
            const int x0 = ox - S + 2 * p, y = oy - S + fy;
            bool okx, oky;
            const int px = tb_wrap(g, 0, x0, okx), py = tb_wrap(g, 1, y, oky);
            int fl = F_USE | (((x0 + y) & 1) ? F_PAR : 0);
            if (okx && oky) fl |= F_VALID;
            if (fy >= S && fy < S + TB_Y && 2 * p >= S && 2 * p < S + TB_X && x0 <= g.n[0] - 2 && y <= g.n[1] - 2)
                fl |= F_OWNED;
            if (2 * p < S - hs) fl |= F_LO;                   // only the odd cell is in the region
            if (2 * p + 1 >= S + TB_X + hs) fl |= F_HI;       // only the even cell is in the region
            sfl[s][k] = fl;
            sq[s][k] = fy * FX + p;
            sxy[s][k] = px + py * s1;
        }
    }
    // input cells of this thread: grid offset (x, y) (-1: outside a wall) and coarse offset
    int ixy[NIN], icxy[NIN];
#pragma unroll
    for (int k = 0; k < NIN; ++k) {
        const int e = tid + k * TB_T;
        ixy[k] = -1;
        icxy[k] = 0;
        if (ZERO || e >= FN) continue;
        const int fy = e / FX, fx = e - fy * FX;
        bool okx, oky;
        const int px = tb_wrap(g, 0, ox - S + fx, okx), py = tb_wrap(g, 1, oy - S + fy, oky);
        if (okx && oky) {
            ixy[k] = px + py * s1;
            icxy[k] = (px + 1) / 2 + ((py + 1) / 2) * int(a.gc.s[1]);
        }
    }

    auto stage_in = [&](int zl) {
        bool okz;
        const int pz = tb_wrap(g, 2, zl, okz);
        float* dst = ring[0][tb_slot(zl)];
        const int cz = ((pz + 1) / 2) * int(a.gc.s[2]);
#pragma unroll
        for (int k = 0; k < NIN; ++k) {
            const int e = tid + k * TB_T;
            if (e >= FN) continue;
            float v = 0.f;
            if (okz && ixy[k] >= 0) {
                v = a.xin[ixy[k] + pz * s2];
                if (a.xc) v += a.xc[icxy[k] + cz];
            }
            const int fy = e / FX, fx = e - fy * FX;
            dst[fy * FX + (fx & 1) * HX + (fx >> 1)] = v;
        }
    };

    const int T0 = z0 - S + 1, T1 = z1 + S - 2;
    if (!ZERO) {
        stage_in(T0 - 1);
        stage_in(T0);
    }
    for (int t = T0; t <= T1; ++t) {
        if (!ZERO) stage_in(t + 1);
        __syncthreads();
#pragma unroll
        for (int s = 0; s < S; ++s) {
            if (t >= T0 + 2 * s) {
                const int zl = t - s;
                const int col = (a.c0 + s) & 1;
                bool okz;
                const int pz = tb_wrap(g, 2, zl, okz);
                const bool own_z = zl >= z0 && zl < z1;
                const int zo = pz * s2;
                float* outp = ZERO ? ring[s < S - 1 ? s : 0][tb_slot(zl)] : ring[s < S - 1 ? s + 1 : 0][tb_slot(zl)];
                const int pin = ZERO ? (s > 0 ? s - 1 : 0) : s;
                const float* pc = ring[pin][tb_slot(zl)];
                const float* pd = ring[pin][tb_slot(zl - 1)];
                const float* pu = ring[pin][tb_slot(zl + 1)];
#pragma unroll
                for (int k = 0; k < 2; ++k) {
                    const int fl = sfl[s][k];
                    if (!(fl & F_USE)) continue;
                    const int e = ((fl & F_PAR ? 1 : 0) + zl + col) & 1;   // which cell of the pair
                    if ((fl & F_LO) && e == 0) continue;
                    if ((fl & F_HI) && e == 1) continue;
                    const int q = sq[s][k] + e * HX;
                    float v = 0.f;
                    if ((fl & F_VALID) && okz) {
                        const int I = sxy[s][k] + e + zo;
                        if (ZERO && s == 0) {
                            v = a.b[I] * a.iD[I];
                        } else {
                            const int qxl = q + (e ? -HX : HX - 1);
                            const float vxl = pc[qxl], vxh = pc[qxl + 1];
                            const float vyl = pc[q - FX], vyh = pc[q + FX];
                            const float vzl = pd[q], vzh = pu[q];
                            float off = L0[I] * vxl + L0[I + 1] * vxh;
                            off += L1[I] * vyl + L1[I + s1] * vyh;
                            off += L2[I] * vzl + L2[I + s2] * vzh;
                            v = (a.b[I] - off) * a.iD[I];
                        }
                        if (s >= S - 2 && (fl & F_OWNED) && own_z) a.xout[I] = v;
                    }
                    if (s < S - 1) outp[q] = v;
                }
            }
            __syncthreads();
        }
    }
}


template <class T, int D>
__global__ void residual_k(Grid g, const T* __restrict__ L, const T* __restrict__ b, const T* __restrict__ xv,
                           T* __restrict__ r) {
    CELL_INTERIOR(g)
    const Nb o = nb_of<D>(g, x, y, z);
    r[I] = b[I] - (off7<D>(g, L, xv, I, o) + diag7<D>(g, L, I) * xv[I]);
}

// residual of the 2^D fine children of each coarse cell, summed straight into the coarse
// right-hand side (residual_k + restrict_k without the fine residual array; same sums, same order)
template <class T, int D, class TL = T>
__global__ void resid_restrict_k(Grid gc, int yc0, int yc1, Grid gf, const TL* __restrict__ L,
                                 const T* __restrict__ b, const T* __restrict__ xv, T* __restrict__ bc) {
    const int xc = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    const int yc = yc0 + int(blockIdx.y * blockDim.y + threadIdx.y);   // coarse rows [yc0, yc1)
    const int zc = D == 3 ? 1 + int(blockIdx.z) : 0;
    if (xc > gc.n[0] - 2 || yc >= yc1) return;
    const int s1 = int(gf.s[1]), s2 = int(gf.s[2]);
    T sum = T(0);
    for (int k = 0; k < (D == 3 ? 2 : 1); ++k)
        for (int j = 0; j < 2; ++j)
            for (int i = 0; i < 2; ++i) {
                const int x = 2 * xc - 1 + i, y = 2 * yc - 1 + j, z = D == 3 ? 2 * zc - 1 + k : 0;
                const int I = x + y * s1 + z * s2;
                const Nb o = nb_of<D>(gf, x, y, z);
                sum += b[I] - (off7<D>(gf, L, xv, I, o) + diag7<D>(gf, L, I) * xv[I]);
            }
    bc[xc + yc * int(gc.s[1]) + zc * int(gc.s[2])] = sum;
}

template <class T>
__global__ void prolong_k(Grid gf, Grid gc, const T* __restrict__ xc, T* __restrict__ xf) {
    const Grid& g = gf;
    INTERIOR_XYZ
    const long long P = lin(gc, (c[0] + 1) / 2, (c[1] + 1) / 2, g.D == 3 ? (c[2] + 1) / 2 : 0);
    xf[I] += xc[P];
}

// Coarsest level: one block, mean-free right-hand side, nuc symmetric red-black sweeps from zero.
template <class T>
__global__ void coarse_k(Grid g, const T* __restrict__ L, const T* __restrict__ iD, T* __restrict__ b,
                         T* __restrict__ xv, int nuc) {
    // the sweeps run on a shared-memory copy of x when the level fits (it holds at most a few
    // hundred cells), with 32-bit cell coordinates
    constexpr int SMAX = 4096;
    __shared__ double red[1024];
    __shared__ T xs[SMAX];
    const int total = int(g.N);
    const bool sm = total <= SMAX;
    T* xw = sm ? xs : xv;
    auto coords = [&](int q, int c[3]) {
        c[0] = q % g.n[0];
        const int r = q / g.n[0];
        c[1] = r % g.n[1];
        c[2] = r / g.n[1];
    };
    double acc = 0.0;
    for (int q = threadIdx.x; q < total; q += blockDim.x) {
        int c[3];
        coords(q, c);
        if (is_interior(g, c)) acc += double(b[q]);
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    long long ninner = 1;
    for (int e = 0; e < g.D; ++e) ninner *= (g.n[e] - 2);
    const T mean = T(red[0] / double(ninner));
    __syncthreads();
    for (int q = threadIdx.x; q < total; q += blockDim.x) {
        int c[3];
        coords(q, c);
        if (is_interior(g, c)) b[q] -= mean;
        xw[q] = T(0);
    }
    __syncthreads();
    for (int it = 0; it < 2 * nuc; ++it) {
        const int color = (it & 1) ^ ((it >> 1) & 1);   // R B, B R, R B, ...
        for (int q = threadIdx.x; q < total; q += blockDim.x) {
            int c[3];
            coords(q, c);
            if (!is_interior(g, c) || ((c[0] + c[1] + c[2]) & 1) != color) continue;
            xw[q] = (b[q] - offdiag(g, L, xw, q, c)) * iD[q];
        }
        __syncthreads();
    }
    if (sm)
        for (int q = threadIdx.x; q < total; q += blockDim.x) xv[q] = xs[q];
}

template <class T>
__global__ void zero_k(long long n, T* a) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
        a[q] = T(0);
}
__global__ void to_f32_k(long long n, const double* __restrict__ a, float* __restrict__ b) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
        b[q] = f32_rn(a[q]);
}
__global__ void to_f64_k(long long n, const float* __restrict__ a, double* __restrict__ b) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
        b[q] = double(a[q]);
}

// ------------------------------------------------------------------ Krylov kernels
// Row loops: a block takes whole x-rows of interior cells (rows dealt round-robin over a
// grid of at most KBLOCKS blocks), so the reductions end in one warp-shuffle block sum per
// block and the cross-block sums read only gridDim.x partials.
constexpr int KTHREADS = 256;
constexpr int KBLOCKS = 1216;   // 8 blocks on each of 152 SMs

// Row loops: block b takes rows b, b + G, b + 2G, ... (G blocks) of the interior; the row's
// (y, z) advance incrementally (a grid holds < 2^31 cells, so 32-bit row numbers suffice)
#define ROWS_FOR(g, DD)                                                                              \
    const int nxi_ = (g).n[0] - 2, nyi_ = (g).n[1] - 2;                                              \
    const int nrows_ = nyi_ * ((DD) == 3 ? (g).n[2] - 2 : 1);                                        \
    const int dy_ = int(gridDim.x) % nyi_, dz_ = int(gridDim.x) / nyi_;                              \
    int y = 1 + int(blockIdx.x) % nyi_, z = ((DD) == 3 ? 1 : 0) + int(blockIdx.x) / nyi_;           \
    for (int rw_ = blockIdx.x; rw_ < nrows_;                                                         \
         rw_ += gridDim.x, y += dy_, z += dz_ + (y > nyi_ ? 1 : 0), y -= (y > nyi_ ? nyi_ : 0))
#define ROWS_BEGIN(g)                                                                      \
    {                                                                                      \
        ROWS_FOR(g, (g).D) {                                                               \
            for (int x = 1 + threadIdx.x; x <= nxi_; x += blockDim.x) {                    \
                [[maybe_unused]] const int c[3] = {x, y, z};                               \
                const long long I = lin(g, x, y, z);
#define ROWS_END \
    }            \
    }            \
    }

// the same with a 32-bit cell index and the dimension fixed at compile time
#define ROWS_BEGIN_D(g)                                                                    \
    {                                                                                      \
        const int s1_ = int((g).s[1]), s2_ = int((g).s[2]);                                \
        ROWS_FOR(g, D) {                                                                   \
            const int row_ = y * s1_ + z * s2_;                                            \
            for (int x = 1 + threadIdx.x; x <= nxi_; x += blockDim.x) {                    \
                const int I = row_ + x;

inline int kblocks(const Grid& g) {
    const long long rows = (long long)(g.n[1] - 2) * (g.D == 3 ? g.n[2] - 2 : 1);
    return int(rows < KBLOCKS ? rows : KBLOCKS);
}

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ unsigned long long warp_max(unsigned long long v) {
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_down_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    return v;
}
// block sums of a and b, valid in thread 0 (fixed order: deterministic)
__device__ __forceinline__ void block_sum2(double& a, double& b) {
    __shared__ double sa[32], sb[32];
    a = warp_sum(a);
    b = warp_sum(b);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) {
        sa[w] = a;
        sb[w] = b;
    }
    __syncthreads();
    if (w == 0) {
        const int nw = blockDim.x >> 5;
        a = warp_sum(lane < nw ? sa[lane] : 0.0);
        b = warp_sum(lane < nw ? sb[lane] : 0.0);
    }
}
__device__ __forceinline__ unsigned long long block_max(unsigned long long m) {
    __shared__ unsigned long long sm[32];
    m = warp_max(m);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) sm[w] = m;
    __syncthreads();
    if (w == 0) m = warp_max(lane < (int)(blockDim.x >> 5) ? sm[lane] : 0ull);
    return m;
}

__device__ __forceinline__ unsigned long long abs_bits(double v) {
    return (unsigned long long)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFull;
}

// diagonal D_I = -Σ_i (L[I,i] + L[I+δi,i]) of the FP64 operator
__device__ __forceinline__ double diag_of(const Grid& g, const double* L, long long I) {
    double dd = 0.0;
    for (int i = 0; i < g.D; ++i) dd -= L[I + i * g.N] + L[I + g.s[i] + i * g.N];
    return dd;
}
// diag_of (same sums, same order) out of line, with scalar arguments, for kernels whose common path
// must not carry its FP64 additions (inlined in a branch of pure arithmetic, the compiler if-converts
// it into every thread)
template <int D>
__device__ __noinline__ double diag_of_cold(const double* L, long long I, long long s1, long long s2, long long N) {
    double dd = 0.0;
    dd -= L[I] + L[I + 1];
    dd -= L[I + N] + L[I + s1 + N];
    if (D == 3) dd -= L[I + 2 * N] + L[I + s2 + 2 * N];
    return dd;
}

__global__ void set_diag64_k(Grid g, const double* __restrict__ L, double* __restrict__ diag) {
    ROWS_BEGIN(g)
    diag[I] = diag_of(g, L, I);
    ROWS_END
}

// Finest-level set-up of the mixed solver in one pass over the FP64 face coefficients L (one
// thread per cell of the ghost-inclusive grid):
//  - the FP32 copy L32 of every coefficient (and its FP16 copy L16, when given), = float(L);
//  - on interior cells the FP64 diagonal D_I = -Σ_i (L[I,i] + L[I+δi,i]) in diag_of's order, and the
//    FP32 inverse diagonal of the FP32 copy with set_diag_k's sums and zero rule.
// Where the 2D coefficients of a cell are bit-identical (pure-phase cells away from walls), the
// FP64 sum ((0 - 2a) - 2a) - 2a (3D; (0 - 2a) - 2a in 2D) is exactly fma(-2D, a, 0): the partial
// sums are exact multiples of a and only the last one rounds, as the fma does; both give +0 for a = ±0.
template <int D>
__global__ void setup_fine_k(Grid g, const double* __restrict__ L, double* __restrict__ diag,
                             float* __restrict__ L32, __half* __restrict__ L16, float* __restrict__ iD32) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = D == 3 ? int(blockIdx.z) : 0;
    if (x >= g.n[0] || y >= g.n[1]) return;
    const long long I = lin(g, x, y, z);
    double a[D];
    float fa[D];
#pragma unroll
    for (int i = 0; i < D; ++i) {
        a[i] = L[I + i * g.N];
        fa[i] = f32_rn(a[i]);
        L32[I + i * g.N] = fa[i];
        if (L16) L16[I + i * g.N] = __float2half_rn(fa[i]);
    }
    if (x < 1 || y < 1 || x > g.n[0] - 2 || y > g.n[1] - 2) return;
    if (D == 3 && (z < 1 || z > g.n[2] - 2)) return;
    double b[D];
    bool same = true;
    const unsigned long long a0 = (unsigned long long)__double_as_longlong(a[0]);
#pragma unroll
    for (int i = 0; i < D; ++i) {
        b[i] = L[I + g.s[i] + i * g.N];
        same = same && (unsigned long long)__double_as_longlong(a[i]) == a0 &&
               (unsigned long long)__double_as_longlong(b[i]) == a0;
    }
    diag[I] = same ? fma(-2.0 * D, a[0], 0.0) : diag_of_cold<D>(L, I, g.s[1], g.s[2], g.N);
    float df = 0.0f;
#pragma unroll
    for (int i = 0; i < D; ++i) df -= fa[i] + f32_rn(b[i]);
    const float eps = 1.1920929e-7f;
    iD32[I] = (df * df < 2.0f * eps) ? 0.0f : 1.0f / df;
}

constexpr int MV_ZT = 8;   // z planes per block of the tiled stencil kernels
inline dim3 mv_tile_grid(const Grid& g) {
    return dim3((g.n[0] - 2 + 31) / 32, (g.n[1] - 2 + 7) / 8, g.D == 3 ? (g.n[2] - 2 + MV_ZT - 1) / MV_ZT : 1);
}

// z_I - D_I x_I - Σ L x_nb as one FMA chain: 2D + 1 FP64 operations where pairwise sums take 3D + 1
// (the residual kernels are bound by the FP64 pipe)
template <int D>
__device__ __forceinline__ double resid_cell(const Grid& g, const double* __restrict__ L, double dd,
                                             const double* __restrict__ zz, const double* __restrict__ xv, int I,
                                             const Nb& o) {
    const int s1 = int(g.s[1]), s2 = int(g.s[2]);
    const double* L1 = L + g.N;
    double v = fma(-dd, xv[I], zz[I]);
    v = fma(-L[I], xv[I + o.xl], v);
    v = fma(-L[I + 1], xv[I + o.xh], v);
    v = fma(-L1[I], xv[I + o.yl], v);
    v = fma(-L1[I + s1], xv[I + o.yh], v);
    if (D == 3) {
        const double* L2 = L1 + g.N;
        v = fma(-L2[I], xv[I + o.zl], v);
        v = fma(-L2[I + s2], xv[I + o.zh], v);
    }
    return v;
}

// r = z - A x over interior cells, L∞(r) into *linf (zeroed by the caller); diag precomputed (or NULL:
// from L).  Row loop over a grid of at most KBLOCKS blocks (no per-block scratch).
template <int D>
__global__ void true_resid_k(Grid g, const double* __restrict__ L, const double* __restrict__ diag,
                             const double* __restrict__ zz, const double* __restrict__ xv, double* __restrict__ r,
                             unsigned long long* linf) {
    unsigned long long m = 0ull;
    ROWS_BEGIN_D(g)
    const Nb o = nb_of<D>(g, x, y, z);
    const double v = resid_cell<D>(g, L, diag ? diag[I] : diag7<D>(g, L, I), zz, xv, I, o);
    r[I] = v;
    const unsigned long long b = abs_bits(v);
    m = b > m ? b : m;
    ROWS_END
    m = block_max(m);
    if (threadIdx.x == 0) atomicMax(linf, m);
}

// The same on the x-y tiles of matvec32_tile_k (32 x 8 cells, MV_ZT z planes per block of 256 threads) with
// the precomputed diagonal; each block's L∞ (as the bit pattern of |r|) into pmax[block], reduced by
// finalize_max_k.
// With r32 given, also the next inner solve's start: r32 = float(r) (integer rounding, no FP64-pipe
// conversion in this FP64-bound kernel) and e32 = 0 on the same interior cells (their ghost entries stay
// zero from the allocation: the whole-array vector updates only ever add zero there).
template <int D>
__global__ void __launch_bounds__(256) true_resid_tile_k(Grid g, const double* __restrict__ L,
                                                         const double* __restrict__ diag,
                                                         const double* __restrict__ zz,
                                                         const double* __restrict__ xv, double* __restrict__ r,
                                                         unsigned long long* __restrict__ pmax,
                                                         float* __restrict__ r32, float* __restrict__ e32) {
    const int x = 1 + int(blockIdx.x) * 32 + int(threadIdx.x & 31), y = 1 + int(blockIdx.y) * 8 + int(threadIdx.x >> 5);
    const int z0 = D == 3 ? 1 + MV_ZT * int(blockIdx.z) : 0;
    unsigned long long m = 0ull;
    auto cell = [&](int z) {
        const int I = x + y * int(g.s[1]) + z * int(g.s[2]);
        const Nb o = nb_of<D>(g, x, y, z);
        const double v = resid_cell<D>(g, L, diag[I], zz, xv, I, o);
        r[I] = v;
        if (r32) {
            r32[I] = f32_rn(v);
            e32[I] = 0.f;
        }
        const unsigned long long b = abs_bits(v);
        m = b > m ? b : m;
    };
    if (x <= g.n[0] - 2 && y <= g.n[1] - 2) {
        if (D == 3 && z0 + MV_ZT - 1 <= g.n[2] - 2) {
#pragma unroll
            for (int k = 0; k < MV_ZT; ++k) cell(z0 + k);   // a full tile (see matvec32_tile_k)
        } else {
            for (int k = 0; k < (D == 3 ? MV_ZT : 1); ++k) {
                if (D == 3 && z0 + k > g.n[2] - 2) break;
                cell(z0 + k);
            }
        }
    }
    m = block_max(m);
    if (threadIdx.x == 0) pmax[blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z)] = m;
}
__global__ void finalize_max_k(const unsigned long long* __restrict__ pmax, long long n, unsigned long long* out) {
    unsigned long long m = 0ull;
    for (long long i = threadIdx.x; i < n; i += blockDim.x) m = pmax[i] > m ? pmax[i] : m;
    m = block_max(m);
    if (threadIdx.x == 0) *out = m;
}

// q = A p and partial dot p·q
template <int D>
__global__ void matvec_dot_k(Grid g, const double* __restrict__ L, const double* __restrict__ diag,
                             const double* __restrict__ pv, double* __restrict__ q, double* __restrict__ partial) {
    double acc = 0.0, unused = 0.0;
    ROWS_BEGIN_D(g)
    const Nb o = nb_of<D>(g, x, y, z);
    const double v = off7<D>(g, L, pv, I, o) + diag[I] * pv[I];
    q[I] = v;
    acc += pv[I] * v;
    ROWS_END
    block_sum2(acc, unused);
    if (threadIdx.x == 0) partial[blockIdx.x] = acc;
}

// partial dots s·q and s·r
__global__ void dot2_k(Grid g, const double* __restrict__ sv, const double* __restrict__ q,
                       const double* __restrict__ r, double* __restrict__ partial) {
    double a1 = 0.0, a2 = 0.0;
    ROWS_BEGIN(g)
    a1 += sv[I] * q[I];
    a2 += sv[I] * r[I];
    ROWS_END
    block_sum2(a1, a2);
    if (threadIdx.x == 0) {
        partial[blockIdx.x] = a1;
        partial[gridDim.x + blockIdx.x] = a2;
    }
}

// fixed-order sum of `n` partials for `k` quantities → out[0..k)
// Σ partial[qd·n + i] over i in a fixed order, valid in thread 0 (a block of 1024 threads)
__device__ double finalize_sum(const double* __restrict__ partial, long long n, int qd) {
    __shared__ double sm[1024];
    double acc = 0.0;
    for (long long i = threadIdx.x; i < n; i += blockDim.x) acc += partial[qd * n + i];
    sm[threadIdx.x] = acc;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sm[threadIdx.x] += sm[threadIdx.x + w];
        __syncthreads();
    }
    const double v = sm[0];
    __syncthreads();
    return v;
}
__global__ void finalize_k(const double* __restrict__ partial, long long n, int k, double* out) {
    for (int qd = 0; qd < k; ++qd) {
        const double v = finalize_sum(partial, n, qd);
        if (threadIdx.x == 0) out[qd] = v;
    }
}
// finalize_sum's value (its 1024 strided partial sums, then its pairwise tree, so the same roundings)
// computed by a block of 256 threads, four strands each; valid in every thread.  sm: 1024 shared doubles.
// Out of line: only the last block of a reduction calls it, and inlined it would raise the streaming
// loop's register count.
__device__ __noinline__ double sum1024_by256(const double* partial, long long n, int qd, double* sm) {
    // the four strands advance together (each still in increasing index order), so that their loads
    // are in flight at the same time
    const double* p = partial + qd * n;
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll 2
    for (long long i0 = threadIdx.x; i0 < n; i0 += 1024) {
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (i0 + 256 * k < n) acc[k] += __ldcg(p + i0 + 256 * k);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) sm[int(threadIdx.x) + 256 * k] = acc[k];
    __syncthreads();
    for (int w = 512; w > 0; w >>= 1) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int v = int(threadIdx.x) + 256 * k;
            if (v < w) sm[v] += sm[v + w];
        }
        __syncthreads();
    }
    const double r = sm[0];
    __syncthreads();
    return r;
}
// After thread 0 of every block has written the block's partials: true in the last block to finish,
// which then sees every partial (each block's write is fenced before its count); the counter is reset
// for the next launch by that block.
__device__ bool last_block(unsigned int* done, unsigned int nblocks) {
    __shared__ bool am_last;
    if (threadIdx.x == 0) {
        __threadfence();
        am_last = atomicAdd(done, 1u) == nblocks - 1;
    }
    __syncthreads();
    if (am_last && threadIdx.x == 0) *done = 0u;
    return am_last;
}
// The inner FCG's scalars on the device, in the host's former FP64 operations: β from s·q and s·r (β = 0
// on the first step), then α = (s·r)/(p·q) with the breakdown test; on a breakdown the update is skipped
// and α, s·r are not carried to the next step.
__device__ void fcg_beta(FcgDev* S, double sq, double sr, int first) {
    const double beta = first ? 0.0 : (-S->alpha_prev * sq) / S->rho_prev;
    S->sr = sr;
    S->beta = beta;
    S->beta32 = float(beta);
}
__device__ void fcg_alpha(FcgDev* S, double pq) {
    const double sr = S->sr;
    const bool stop = !(pq != 0.0) || !isfinite(pq) || !isfinite(sr) || !isfinite(S->beta);
    const double alpha = sr / pq;
    S->alpha32 = float(alpha);
    S->stop = stop ? 1 : 0;
    S->rin = 0u;
    if (!stop) {
        S->rho_prev = sr;
        S->alpha_prev = alpha;
    }
}

__global__ void xpby_k(Grid g, const double* __restrict__ sv, double beta, double* __restrict__ pv) {
    ROWS_BEGIN(g)
    pv[I] = (beta == 0.0) ? sv[I] : sv[I] + beta * pv[I];
    ROWS_END
}

// x += α p ; r -= α q ; L∞(r)
__global__ void update_k(Grid g, double alpha, const double* __restrict__ pv, const double* __restrict__ q,
                         double* __restrict__ xv, double* __restrict__ r, unsigned long long* linf) {
    unsigned long long m = 0ull;
    ROWS_BEGIN(g)
    xv[I] += alpha * pv[I];
    const double v = r[I] - alpha * q[I];
    r[I] = v;
    const unsigned long long b = abs_bits(v);
    m = b > m ? b : m;
    ROWS_END
    m = block_max(m);
    if (threadIdx.x == 0) atomicMax(linf, m);
}

// ---- FP32 inner Krylov kernels (mixed / learned): FP32 products, per-thread sums in FP32
// over its cells, FP64 block and cross-block sums.
// q = A p and per-block partial sums of p·q on x-y tiles: a block of 256 threads takes 32 x 8 cells of
// MV_ZT consecutive z planes (one plane in 2D), so that the stencil's x and y neighbours come from L1 and
// every load of a cell issues at once (a row loop, one row per block and step, waits for each row's
// loads and fetches the y neighbours from other SMs' rows through L2).  The partials, one per block,
// are summed in a fixed order.  Four blocks per SM (64 registers) let a thread keep more of its planes'
// loads in flight: 0.180 against 0.194 ms per launch at 256x512x256 with the default 32 registers.

template <int D>
__global__ void __launch_bounds__(256, 4) matvec32_tile_k(Grid g, const float* __restrict__ L,
                                                       const float* __restrict__ pv, float* __restrict__ q,
                                                       double* __restrict__ partial, FcgDev* S) {
    const int x = 1 + int(blockIdx.x) * 32 + int(threadIdx.x & 31), y = 1 + int(blockIdx.y) * 8 + int(threadIdx.x >> 5);
    const int z0 = D == 3 ? 1 + MV_ZT * int(blockIdx.z) : 0;
    float acc = 0.f;
    auto cell = [&](int z) {
        const int I = x + y * int(g.s[1]) + z * int(g.s[2]);
        const Nb o = nb_of<D>(g, x, y, z);
        const float v = off7<D>(g, L, pv, I, o) + diag7<D>(g, L, I) * pv[I];
        q[I] = v;
        acc += pv[I] * v;
    };
    if (x <= g.n[0] - 2 && y <= g.n[1] - 2) {
        if (D == 3 && z0 + MV_ZT - 1 <= g.n[2] - 2) {
            // a full tile: no bound test between the planes, so that their loads can be issued early
            // and a plane's values reused as the next plane's z neighbours
#pragma unroll
            for (int k = 0; k < MV_ZT; ++k) cell(z0 + k);
        } else {
            for (int k = 0; k < (D == 3 ? MV_ZT : 1); ++k) {
                if (D == 3 && z0 + k > g.n[2] - 2) break;
                cell(z0 + k);
            }
        }
    }
    // the warp's sum in FP32 (a fixed shuffle tree), the block's eight warp sums in FP64 by one thread:
    // a per-thread FP64 reduction costs more FP64-pipe time than the stencil itself
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    __shared__ double ws[8];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = double(acc);
    __syncthreads();
    const unsigned int nb = gridDim.x * gridDim.y * gridDim.z;
    if (threadIdx.x == 0) {
        double a = 0.0;
        for (int w = 0; w < 8; ++w) a += ws[w];
        partial[blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z)] = a;
    }
    // the last block: p·q in a fixed order, then α
    if (!last_block(&S->done_mv, nb)) return;
    __shared__ double sm[1024];
    const double pq = sum1024_by256(partial, nb, 0, sm);
    if (threadIdx.x == 0) fcg_alpha(S, pq);
}

// Whole-array FP32 vector kernels of the inner solve.  Only interior cells of these vectors are
// ever written, so their ghost entries stay zero and sums and updates over all N entries equal
// those over the interior; the arrays are streamed as 16-byte vectors (cudaMalloc alignment),
// the N mod 4 tail by the first threads.
__global__ void dot2_32_k(long long n, const float* __restrict__ sv, const float* __restrict__ q,
                          const float* __restrict__ r, double* __restrict__ partial, FcgDev* S, int first) {
    float a1 = 0.f, a2 = 0.f;
    const long long n4 = n / 4, stride = (long long)gridDim.x * blockDim.x;
    const long long t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const float4* s4 = reinterpret_cast<const float4*>(sv);
    const float4* q4 = reinterpret_cast<const float4*>(q);
    const float4* r4 = reinterpret_cast<const float4*>(r);
    for (long long i = t0; i < n4; i += stride) {
        const float4 a = s4[i], bq = q4[i], br = r4[i];
        a1 += a.x * bq.x + a.y * bq.y + a.z * bq.z + a.w * bq.w;
        a2 += a.x * br.x + a.y * br.y + a.z * br.z + a.w * br.w;
    }
    if (t0 < n - 4 * n4) {
        const long long i = 4 * n4 + t0;
        a1 += sv[i] * q[i];
        a2 += sv[i] * r[i];
    }
    double b1 = a1, b2 = a2;
    block_sum2(b1, b2);
    if (threadIdx.x == 0) {
        partial[blockIdx.x] = b1;
        partial[gridDim.x + blockIdx.x] = b2;
    }
    // the last block: s·q and s·r in a fixed order, then β
    if (!last_block(&S->done_dot, gridDim.x)) return;
    __shared__ double sm[1024];
    const double sq = sum1024_by256(partial, gridDim.x, 0, sm);
    const double sr = sum1024_by256(partial, gridDim.x, 1, sm);
    if (threadIdx.x == 0) fcg_beta(S, sq, sr, first);
}

// p = s + β p; β = 0 restarts from s without reading the old direction (which a rejected
// preconditioner output may have left non-finite)
__global__ void xpby32_k(long long n, const float* __restrict__ sv, const FcgDev* __restrict__ S,
                         float* __restrict__ pv) {
    const float beta = S->beta32;
    const long long n4 = n / 4, stride = (long long)gridDim.x * blockDim.x;
    const long long t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const float4* s4 = reinterpret_cast<const float4*>(sv);
    float4* p4 = reinterpret_cast<float4*>(pv);
    const bool restart = beta == 0.f;
    for (long long i = t0; i < n4; i += stride) {
        const float4 a = s4[i];
        if (restart) {
            p4[i] = a;
        } else {
            const float4 p = p4[i];
            p4[i] = make_float4(a.x + beta * p.x, a.y + beta * p.y, a.z + beta * p.z, a.w + beta * p.w);
        }
    }
    if (t0 < n - 4 * n4) {
        const long long i = 4 * n4 + t0;
        pv[i] = restart ? sv[i] : sv[i] + beta * pv[i];
    }
}

// e += α p ; r -= α q ; L∞(r) as float bits into S->rin (nothing after a breakdown)
__global__ void update32_k(long long n, FcgDev* __restrict__ S, const float* __restrict__ pv,
                           const float* __restrict__ q, float* __restrict__ e, float* __restrict__ r) {
    if (S->stop) return;
    const float alpha = S->alpha32;
    unsigned int* linf = &S->rin;
    unsigned long long m = 0ull;
    const long long n4 = n / 4, stride = (long long)gridDim.x * blockDim.x;
    const long long t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const float4* p4 = reinterpret_cast<const float4*>(pv);
    const float4* q4 = reinterpret_cast<const float4*>(q);
    float4* e4 = reinterpret_cast<float4*>(e);
    float4* r4 = reinterpret_cast<float4*>(r);
    auto mx = [&](float v) {
        const unsigned long long b = __float_as_uint(v) & 0x7FFFFFFFu;
        m = b > m ? b : m;
    };
    for (long long i = t0; i < n4; i += stride) {
        const float4 p = p4[i], qq = q4[i];
        float4 ee = e4[i], rr = r4[i];
        ee.x += alpha * p.x; ee.y += alpha * p.y; ee.z += alpha * p.z; ee.w += alpha * p.w;
        rr.x -= alpha * qq.x; rr.y -= alpha * qq.y; rr.z -= alpha * qq.z; rr.w -= alpha * qq.w;
        e4[i] = ee;
        r4[i] = rr;
        mx(rr.x); mx(rr.y); mx(rr.z); mx(rr.w);
    }
    if (t0 < n - 4 * n4) {
        const long long i = 4 * n4 + t0;
        e[i] += alpha * pv[i];
        const float v = r[i] - alpha * q[i];
        r[i] = v;
        mx(v);
    }
    m = block_max(m);
    if (threadIdx.x == 0) atomicMax(linf, (unsigned int)m);
}

// ---- learned hybrid preconditioner: partial dots n·t and n·An for the energy-optimal step
// ω = (n·t)/(n·An), which minimises the A-norm of the error e - ω n left behind the V-cycle
// (t = A e); A is negative semi-definite here, so both dots carry the same sign.
template <int D>
__global__ void energy_dots_k(Grid g, const float* __restrict__ L, const float* __restrict__ n,
                              const float* __restrict__ t, double* __restrict__ partial) {
    float a1 = 0.f, a2 = 0.f;
    ROWS_BEGIN_D(g)
    const Nb o = nb_of<D>(g, x, y, z);
    const float an = off7<D>(g, L, n, I, o) + diag7<D>(g, L, I) * n[I];
    a1 += n[I] * t[I];
    a2 += n[I] * an;
    ROWS_END
    double b1 = a1, b2 = a2;
    block_sum2(b1, b2);
    if (threadIdx.x == 0) {
        partial[blockIdx.x] = b1;
        partial[gridDim.x + blockIdx.x] = b2;
    }
}

// s += ω n with ω = (n·t)/(n·An) from the device dots (0 unless both are finite and n·An ≠ 0)
__global__ void add_scaled_k(Grid g, const double* __restrict__ dots, const float* __restrict__ nv,
                             float* __restrict__ sv) {
    const double tn = dots[0], nan_ = dots[1];
    const bool ok = nan_ != 0.0 && nan_ == nan_ && tn == tn && fabs(nan_) < 1e300 && fabs(tn) < 1e300;
    const float w = float(ok ? tn / nan_ : 0.0);
    ROWS_BEGIN(g)
    sv[I] += w * nv[I];
    ROWS_END
}

// x += e (FP64 += FP32), interior cells
// double(v) with integer operations for zeros, normal numbers, inf and NaN (the conversion instruction
// issues on the FP64 pipe); FP32 subnormals take the conversion, out of line
__device__ __noinline__ double widen_cold(float v) { return double(v); }
__device__ __forceinline__ double widen_exact(float v) {
    const unsigned b = __float_as_uint(v);
    return (((b >> 23) & 0xFFu) != 0u || (b << 1) == 0u) ? ff_widen(v) : widen_cold(v);
}

// x += e over interior cells, on the tiles of matvec32_tile_k (one cell per thread and plane)
template <int D>
__global__ void __launch_bounds__(256) add_correction_k(Grid g, const float* __restrict__ e, double* __restrict__ xv) {
    const int x = 1 + int(blockIdx.x) * 32 + int(threadIdx.x & 31), y = 1 + int(blockIdx.y) * 8 + int(threadIdx.x >> 5);
    const int z0 = D == 3 ? 1 + MV_ZT * int(blockIdx.z) : 0;
    if (x > g.n[0] - 2 || y > g.n[1] - 2) return;
#pragma unroll
    for (int k = 0; k < (D == 3 ? MV_ZT : 1); ++k) {
        const int z = z0 + k;
        if (D == 3 && z > g.n[2] - 2) break;
        const int I = x + y * int(g.s[1]) + z * int(g.s[2]);
        xv[I] += widen_exact(e[I]);
    }
}

// periodic ghosts of a scalar (WaterLily perBC!), one thread per cell of the boundary planes
__global__ void perbc_k(Grid g, double* a) {
    int c[3];
    if (!bc_plane_cell(g, blockIdx.x * (long long)blockDim.x + threadIdx.x, c)) return;
    const int x = c[0], y = c[1], z = c[2];
    bool any = false;
    for (int e = 0; e < g.D; ++e)
        if (g.isper(e) && (c[e] == 0 || c[e] == g.n[e] - 1)) {
            c[e] = bc_src(g, e, c[e]);
            any = true;
        }
    if (!any) return;
    // only read positions that no thread writes: the mapped position must have
    // no periodic ghost coordinate left (it has none after mapping)
    a[lin(g, x, y, z)] = a[lin3(g, c)];
}

}  // namespace

// ------------------------------------------------------------------ host side

// z-planes per block of the blocked smoother: about eight blocks per multiprocessor in all,
// each block marching at least 4 S planes
static int tb_zchunk(const Grid& g, int S, int nsm) {
    const int tiles = ((g.n[0] - 2 + TB_X - 1) / TB_X) * ((g.n[1] - 2 + TB_Y - 1) / TB_Y);
    const int nzi = g.n[2] - 2;
    const int want = std::max(1, (8 * std::max(nsm, 1)) / std::max(tiles, 1));
    int zc = (nzi + want - 1) / want;
    zc = std::max(zc, std::min(nzi, 4 * S));
    return std::max(zc, 1);
}

// the blocked smoother runs the FP32 V-cycle of a 3D level with an even number of interior
// cells in every dimension (every level but the coarsest), for nu1, nu2 in {1, 2}
static bool tb_usable(const PoissonMG* mg, const Grid& g) {
    if (mg->smoother != IA_SMOOTHER_BLOCKED || g.D != 3 || mg->omega != 1.0) return false;
    if (mg->nu1 < 1 || mg->nu1 > 2 || mg->nu2 < 1 || mg->nu2 > 2) return false;
    for (int e = 0; e < 3; ++e)
        if ((g.n[e] - 2) % 2 != 0) return false;
    return true;
}

static void tb_launch(const PoissonMG* mg, const TbArgs& a, int S, cudaStream_t st) {
    TbArgs b = a;
    b.zchunk = tb_zchunk(a.g, S, mg->nsm);
    const dim3 grid((a.g.n[0] - 2 + TB_X - 1) / TB_X, (a.g.n[1] - 2 + TB_Y - 1) / TB_Y,
                    (a.g.n[2] - 2 + b.zchunk - 1) / b.zchunk);
    const bool zero = a.xin == nullptr;
    if (S == 4) {
        if (zero) rbgs_tb_k<4, true><<<grid, TB_T, 0, st>>>(b);
        else rbgs_tb_k<4, false><<<grid, TB_T, 0, st>>>(b);
    } else {
        if (zero) rbgs_tb_k<2, true><<<grid, TB_T, 0, st>>>(b);
        else rbgs_tb_k<2, false><<<grid, TB_T, 0, st>>>(b);
    }
    ia::note_launch();
}

template <class T>
static cudaError_t vcycle(ia_handle* h, PoissonMG* mg, int l, cudaStream_t st, int nu1, int nu2, int nuc) {
    auto& L = mg->lev[l];
    T* x = L.template x_<T>();
    T* b = L.template b_<T>();
    const T* Lc = L.template L_<T>();
    const T* iD = L.template iD_<T>();
    if (l == mg->nlev - 1) {
        { coarse_k<T><<<1, 1024, 0, st>>>(L.g, Lc, iD, b, x, nuc); ia::note_launch(); }
        return cudaGetLastError();
    }
    if constexpr (sizeof(T) == 4) {
        if (tb_usable(mg, L.g)) {
            // pre-smoothing from zero into the level's scratch vector, residual restriction
            // from it, then post-smoothing of scratch + prolongated correction into x
            auto& C = mg->lev[l + 1];
            TbArgs ta;
            ta.g = L.g;
            ta.gc = C.g;
            ta.L = Lc;
            ta.b = b;
            ta.iD = iD;
            ta.xin = nullptr;
            ta.xc = nullptr;
            ta.xout = L.r32;
            ta.c0 = 0;
            ta.zchunk = 1;
            int tk = (l == 0) ? timing_begin(h, TK_MG_FINE) : -1;
            tb_launch(mg, ta, 2 * nu1, st);
            timing_end(h, tk);
            { resid_restrict_k<T, 3><<<cell_grid(C.g), blk(), 0, st>>>(C.g, 1, C.g.n[1] - 1, L.g, Lc, b, L.r32, C.template b_<T>()); ia::note_launch(); }
            cudaError_t e = vcycle<T>(h, mg, l + 1, st, nu1, nu2, nuc);
            if (e != cudaSuccess) return e;
            ta.xin = L.r32;
            ta.xc = C.x32;
            ta.xout = x;
            ta.c0 = 1;
            tk = (l == 0) ? timing_begin(h, TK_MG_FINE) : -1;
            tb_launch(mg, ta, 2 * nu2, st);
            timing_end(h, tk);
            return cudaGetLastError();
        }
    }
    // the finest level may smooth a different number of times than the coarser ones (ia_poisson_mg_fine);
    // the recursion below passes the coarse counts on
    const int nu1_here = (l == 0 && mg->nu1f > 0) ? mg->nu1f : nu1;
    const int nu2_here = (l == 0 && mg->nu2f > 0) ? mg->nu2f : nu2;
    // the finest mixed level's half-sweeps and residual restriction read the FP16 coefficient copy
    const __half* L16 = nullptr;
    if constexpr (sizeof(T) == 4) L16 = (l == 0 && mg->coef16) ? L.L16 : nullptr;
    auto& C = mg->lev[l + 1];
    const T om = T(mg->omega);
    // each launch takes the interior rows [y0, y1)
    auto rows = [](dim3 gr, int y0, int y1) {
        gr.y = unsigned((y1 - y0 + 7) / 8);
        return gr;
    };
    auto half = [&](int color, int y0, int y1) {
        const int tk = (l == 0) ? timing_begin(h, TK_MG_FINE) : -1;
        const dim3 gr = rows(pair_tile_grid(L.g), y0, y1);
        if (L16) {
            if (L.g.D == 3) rbgs_pair_k<T, 3, false, __half><<<gr, blk(), 0, st>>>(L.g, y0, y1, L16, b, x, color, om);
            else rbgs_pair_k<T, 2, false, __half><<<gr, blk(), 0, st>>>(L.g, y0, y1, L16, b, x, color, om);
        } else {
            if (L.g.D == 3) rbgs_pair_k<T, 3><<<gr, blk(), 0, st>>>(L.g, y0, y1, Lc, b, x, color, om);
            else rbgs_pair_k<T, 2><<<gr, blk(), 0, st>>>(L.g, y0, y1, Lc, b, x, color, om);
        }
        ia::note_launch();
        timing_end(h, tk);
    };
    // the relaxed first red half-sweep of a post-smoothing: the red cells still hold x without the
    // coarse correction, which it adds to the value it reads
    auto half_prol = [&](int y0, int y1) {
        const int tk = (l == 0) ? timing_begin(h, TK_MG_FINE) : -1;
        const dim3 gr = rows(pair_tile_grid(L.g), y0, y1);
        const T* xc = C.template x_<T>();
        if (L16 && L.g.D == 3) rbgs_pair_k<T, 3, true, __half><<<gr, blk(), 0, st>>>(L.g, y0, y1, L16, b, x, 0, om, C.g, xc);
        else if (L16) rbgs_pair_k<T, 2, true, __half><<<gr, blk(), 0, st>>>(L.g, y0, y1, L16, b, x, 0, om, C.g, xc);
        else if (L.g.D == 3) rbgs_pair_k<T, 3, true><<<gr, blk(), 0, st>>>(L.g, y0, y1, Lc, b, x, 0, om, C.g, xc);
        else rbgs_pair_k<T, 2, true><<<gr, blk(), 0, st>>>(L.g, y0, y1, Lc, b, x, 0, om, C.g, xc);
        ia::note_launch();
        timing_end(h, tk);
    };
    // over-relaxed updates read the cell's own previous value: the red values of the first sweep
    // are then stored, and the post-smoothing's first red half-sweep adds the coarse correction
    // to the value it reads
    const bool relax = mg->omega != 1.0;
    const int write_red = (nu1_here == 1 || relax) ? 1 : 0;
    // first black half-sweep: from x = 0 (pre) or from x + P(x_coarse) (post)
    auto first = [&](bool prol, int y0, int y1) {
        const int tk = (l == 0) ? timing_begin(h, TK_MG_FIRST) : -1;
        const dim3 gr = rows(pair_grid(L.g), y0, y1);
        const T* xc = C.template x_<T>();
        const int wr = prol ? 0 : write_red;
        if (L16 && L.g.D == 3) {
            if (prol) rbgs_first_k<T, 3, true, __half><<<gr, blk(), 0, st>>>(L.g, y0, y1, C.g, L16, b, iD, xc, x, wr, om);
            else rbgs_first_k<T, 3, false, __half><<<gr, blk(), 0, st>>>(L.g, y0, y1, C.g, L16, b, iD, xc, x, wr, om);
        } else if (L16) {
            if (prol) rbgs_first_k<T, 2, true, __half><<<gr, blk(), 0, st>>>(L.g, y0, y1, C.g, L16, b, iD, xc, x, wr, om);
            else rbgs_first_k<T, 2, false, __half><<<gr, blk(), 0, st>>>(L.g, y0, y1, C.g, L16, b, iD, xc, x, wr, om);
        } else if (L.g.D == 3) {
            if (prol) rbgs_first_k<T, 3, true><<<gr, blk(), 0, st>>>(L.g, y0, y1, C.g, Lc, b, iD, xc, x, wr, om);
            else rbgs_first_k<T, 3, false><<<gr, blk(), 0, st>>>(L.g, y0, y1, C.g, Lc, b, iD, xc, x, wr, om);
        } else {
            if (prol) rbgs_first_k<T, 2, true><<<gr, blk(), 0, st>>>(L.g, y0, y1, C.g, Lc, b, iD, xc, x, wr, om);
            else rbgs_first_k<T, 2, false><<<gr, blk(), 0, st>>>(L.g, y0, y1, C.g, Lc, b, iD, xc, x, wr, om);
        }
        ia::note_launch();
        timing_end(h, tk);
    };
    // residual restriction of the coarse rows [yc0, yc1)
    auto restrict_rows = [&](int yc0, int yc1) {
        const dim3 gr = rows(cell_grid(C.g), yc0, yc1);
        T* bc = C.template b_<T>();
        if (L16 && L.g.D == 3) resid_restrict_k<T, 3, __half><<<gr, blk(), 0, st>>>(C.g, yc0, yc1, L.g, L16, b, x, bc);
        else if (L16) resid_restrict_k<T, 2, __half><<<gr, blk(), 0, st>>>(C.g, yc0, yc1, L.g, L16, b, x, bc);
        else if (L.g.D == 3) resid_restrict_k<T, 3><<<gr, blk(), 0, st>>>(C.g, yc0, yc1, L.g, Lc, b, x, bc);
        else resid_restrict_k<T, 2><<<gr, blk(), 0, st>>>(C.g, yc0, yc1, L.g, Lc, b, x, bc);
        ia::note_launch();
    };
    // A smoothing is a chain of stages, each a half-sweep of one colour that reads the previous
    // stage's values in rows y-1 .. y+1 (and its own colour's values from two stages back).  On the
    // finest FP32 level with walls in y, the chain runs as a wavefront over slabs of slab_rows rows:
    // for slab k the stage s takes rows [a_k - s, a_(k+1) - s), one row behind stage s-1, so every row
    // a stage reads is final for its predecessor and not yet rewritten by its successor (red-black
    // updates read only the other colour).  The results are those of whole-level half-sweeps, bit for
    // bit, while a slab's rows are still in L2 for the next stage.  The restriction follows with the
    // coarse rows whose fine rows (and their neighbours) are final.
    const bool slab = sizeof(T) == 4 && l == 0 && mg->slab_rows > 0 && L.g.D == 3 && !L.g.isper(1) &&
                      L.g.n[1] - 2 > mg->slab_rows;
    auto chain = [&](int S, auto&& stage, bool with_restrict) {
        const int ny = L.g.n[1] - 2, yend = L.g.n[1] - 1;
        const int R = slab ? std::max(mg->slab_rows, 2 * S) : ny;
        const int K = (ny + R - 1) / R;
        int yc_done = 1;
        for (int k = 0; k < K; ++k) {
            const bool lastk = k + 1 == K;
            const int a0 = 1 + k * R, a1 = lastk ? yend : 1 + (k + 1) * R;
            for (int s = 0; s < S; ++s) {
                const int y0 = (k == 0) ? 1 : a0 - s, y1 = lastk ? yend : a1 - s;
                if (y1 > y0) stage(s, y0, y1);
            }
            if (with_restrict) {
                const int yc1 = lastk ? C.g.n[1] - 1 : std::min(C.g.n[1] - 1, (a1 - S - 1) / 2 + 1);
                if (yc1 > yc_done) {
                    restrict_rows(yc_done, yc1);
                    yc_done = yc1;
                }
            }
        }
    };
    // pre-smoothing: first (black with the red values in place), then (red, black) nu1 - 1 times
    chain(2 * nu1_here - 1, [&](int s, int y0, int y1) {
        if (s == 0) first(false, y0, y1);
        else half((s & 1) ? 0 : 1, y0, y1);
    }, true);
    cudaError_t e = vcycle<T>(h, mg, l + 1, st, nu1, nu2, nuc);
    if (e != cudaSuccess) return e;
    if (nu2_here == 0) {
        { prolong_k<T><<<grd(L.g), blk(), 0, st>>>(L.g, C.g, C.template x_<T>(), x); ia::note_launch(); }
        return cudaGetLastError();
    }
    // post-smoothing: first (black from x + P(x_coarse)), red (adding the correction when relaxed),
    // then (black, red) nu2 - 1 times
    chain(2 * nu2_here, [&](int s, int y0, int y1) {
        if (s == 0) first(true, y0, y1);
        else if (s == 1 && relax) half_prol(y0, y1);
        else half((s & 1) ? 0 : 1, y0, y1);
    }, false);
    return cudaGetLastError();
}

// The finest-level V-cycle through its CUDA graph (plain launches while per-launch timing is on)
template <class T>
static cudaError_t vcycle_run(ia_handle* h, PoissonMG* mg, cudaStream_t st) {
    if (h->timing.on) return vcycle<T>(h, mg, 0, st, mg->nu1, mg->nu2, mg->nuc);
    const int k = sizeof(T) == 4 ? 0 : 1;
    int* nu = mg->vgraph_nu[k];
    if (mg->vgraph[k] && (nu[0] != mg->nu1 || nu[1] != mg->nu2 || nu[2] != mg->nuc || nu[3] != mg->smoother ||
                          mg->vgraph_omega[k] != mg->omega || mg->vgraph_c16[k] != mg->coef16 ||
                          mg->vgraph_slab[k] != mg->slab_rows || mg->vgraph_fine[k] != mg->nu1f * 64 + mg->nu2f)) {
        cudaGraphExecDestroy(mg->vgraph[k]);
        mg->vgraph[k] = nullptr;
    }
    if (!mg->vgraph[k]) {
        if (!mg->capture && cudaStreamCreateWithFlags(&mg->capture, cudaStreamNonBlocking) != cudaSuccess)
            return vcycle<T>(h, mg, 0, st, mg->nu1, mg->nu2, mg->nuc);
        const long long n0 = launch_count();
        cudaGraph_t gr = nullptr;
        cudaError_t e = cudaStreamBeginCapture(mg->capture, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            const cudaError_t ek = vcycle<T>(h, mg, 0, mg->capture, mg->nu1, mg->nu2, mg->nuc);
            e = cudaStreamEndCapture(mg->capture, &gr);
            if (e == cudaSuccess) e = ek;
        }
        const long long captured = launch_count() - n0;
        note_launches(-captured);   // captured, not launched
        if (e == cudaSuccess) e = cudaGraphInstantiate(&mg->vgraph[k], gr, 0);
        if (gr) cudaGraphDestroy(gr);
        if (e != cudaSuccess) {
            mg->vgraph[k] = nullptr;
            cudaGetLastError();
            return vcycle<T>(h, mg, 0, st, mg->nu1, mg->nu2, mg->nuc);
        }
        mg->vgraph_kernels[k] = captured;
        nu[0] = mg->nu1;
        nu[1] = mg->nu2;
        nu[2] = mg->nuc;
        nu[3] = mg->smoother;
        mg->vgraph_omega[k] = mg->omega;
        mg->vgraph_c16[k] = mg->coef16;
        mg->vgraph_slab[k] = mg->slab_rows;
        mg->vgraph_fine[k] = mg->nu1f * 64 + mg->nu2f;
    }
    note_launches(mg->vgraph_kernels[k]);
    return cudaGraphLaunch(mg->vgraph[k], st);
}

// the finest-level coefficients L = 1/ρ_face lie in [1/max(λρ,1), 1/min(λρ,1)] (0 on wall faces): FP16
// holds them (relative precision 2^-11) when that interval lies inside its normal range
bool coef16_fits(double lrho) {
    const double lo = lrho < 1.0 ? lrho : 1.0, hi = lrho < 1.0 ? 1.0 : lrho;
    return lo > 0.0 && 1.0 / lo <= 60000.0 && 1.0 / hi >= 1e-4;
}

// Rows per slab of the finest-level wavefront: the bytes a stage touches per interior row (x, b, the
// inverse diagonal and the coefficients) times the rows of a slab within about 3/5 of L2, a multiple of
// 8 rows (measured at 256x512x256: 64 rows 45.7 ms per step, 32 rows 47.0, 16 rows 49.9, whole-level
// half-sweeps 46.3: smaller slabs lose more to launches and partial blocks than they gain in L2 hits).
// 0 (whole-level half-sweeps) where the wavefront does not apply.
int mg_create(ia_handle* h) {
    PoissonMG* mg = new PoissonMG();
    h->mg = mg;
    const Grid& g0 = h->g;
    long long Nint[3] = {g0.n[0] - 2, g0.n[1] - 2, g0.D == 3 ? g0.n[2] - 2 : 1};
    const bool mixed = h->cfg.poisson_mode != IA_POISSON_FP64;
    mg->coef16 = (mixed && coef16_fits(h->cfg.lrho)) ? 1 : 0;
    int nl = 0;
    while (nl < MG_MAX_LEVELS) {
        int64_t N[3] = {Nint[0], Nint[1], Nint[2]};
        MGLevel& L = mg->lev[nl];
        L.g = make_grid(g0.D, g0.per, N);
        const size_t n = (size_t)L.g.N;
        cudaError_t e = cudaSuccess;
        // FP64 levels always exist for level 0 (fine operator copies) and for the FP64 mode
        if (!mixed) {
            e = e ? e : cudaMalloc(&L.x, 8 * n);
            e = e ? e : cudaMalloc(&L.b, 8 * n);
            e = e ? e : cudaMalloc(&L.r, 8 * n);
            e = e ? e : cudaMalloc(&L.L, 8 * n * g0.D);
            e = e ? e : cudaMalloc(&L.iD, 8 * n);
            if (!e) {
                cudaMemset(L.x, 0, 8 * n);
                cudaMemset(L.b, 0, 8 * n);
                cudaMemset(L.r, 0, 8 * n);
                cudaMemset(L.iD, 0, 8 * n);
                cudaMemset(L.L, 0, 8 * n * g0.D);
            }
        } else {
            e = e ? e : cudaMalloc(&L.x32, 4 * n);
            e = e ? e : cudaMalloc(&L.b32, 4 * n);
            e = e ? e : cudaMalloc(&L.r32, 4 * n);
            e = e ? e : cudaMalloc(&L.L32, 4 * n * g0.D);
            e = e ? e : cudaMalloc(&L.iD32, 4 * n);
            if (nl == 0) e = e ? e : cudaMalloc(&L.L16, 2 * n * g0.D);
            if (!e) {
                cudaMemset(L.x32, 0, 4 * n);
                cudaMemset(L.b32, 0, 4 * n);
                cudaMemset(L.r32, 0, 4 * n);
                cudaMemset(L.iD32, 0, 4 * n);
                cudaMemset(L.L32, 0, 4 * n * g0.D);
            }
        }
        if (e != cudaSuccess) return IA_ERR_CUDA;
        ++nl;
        bool can = true;
        for (int d = 0; d < g0.D; ++d)
            if (Nint[d] % 2 != 0 || Nint[d] < 4) can = false;
        long long cells = 1;
        for (int d = 0; d < g0.D; ++d) cells *= Nint[d];
        if (!can || cells <= 512) break;
        for (int d = 0; d < g0.D; ++d) Nint[d] /= 2;
    }
    mg->nlev = nl;
    const size_t N = (size_t)g0.N;
    cudaError_t e = cudaSuccess;
    e = e ? e : cudaMalloc(&mg->r, 8 * N);
    e = e ? e : cudaMalloc(&mg->s, 8 * N);
    e = e ? e : cudaMalloc(&mg->p, 8 * N);
    e = e ? e : cudaMalloc(&mg->q, 8 * N);
    mg->kb = kblocks(g0);
    {
        const dim3 mv = mv_tile_grid(g0);
        mg->mvb = (long long)mv.x * mv.y * mv.z;
    }
    e = e ? e : cudaMalloc(&mg->partial, 8 * std::max<size_t>(2 * (size_t)KBLOCKS, (size_t)mg->mvb));
    e = e ? e : cudaMalloc(&mg->diag64, 8 * N);
    if (!e) cudaMemset(mg->diag64, 0, 8 * N);
    if (mixed) {
        e = e ? e : cudaMalloc(&mg->p32, 4 * N);
        e = e ? e : cudaMalloc(&mg->q32, 4 * N);
        e = e ? e : cudaMalloc(&mg->e32, 4 * N);
        if (!e) {
            cudaMemset(mg->p32, 0, 4 * N);
            cudaMemset(mg->q32, 0, 4 * N);
            cudaMemset(mg->e32, 0, 4 * N);
        }
    }
    if (h->cfg.poisson_mode == IA_POISSON_LEARNED) {
        e = e ? e : cudaMalloc(&mg->rl32, 4 * N);
        e = e ? e : cudaMalloc(&mg->nl32, 4 * N);
        e = e ? e : cudaMalloc(&mg->t32, 4 * N);
        if (!e) {   // ghosts stay zero: only interior cells are written
            cudaMemset(mg->rl32, 0, 4 * N);
            cudaMemset(mg->nl32, 0, 4 * N);
            cudaMemset(mg->t32, 0, 4 * N);
        }
    }
    e = e ? e : cudaMalloc(&mg->dsc, 8 * 16);
    e = e ? e : cudaMalloc(&mg->fcg, sizeof(FcgDev));
    if (!e) cudaMemset(mg->fcg, 0, sizeof(FcgDev));
    e = e ? e : cudaMallocHost(&mg->hsc, 8 * 16);
    if (e != cudaSuccess) return IA_ERR_CUDA;
    cudaMemset(mg->r, 0, 8 * N);
    cudaMemset(mg->s, 0, 8 * N);
    cudaMemset(mg->p, 0, 8 * N);
    cudaMemset(mg->q, 0, 8 * N);
    mg->nu1 = 2;
    mg->nu2 = 2;
    mg->nuc = 16;
    {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&mg->nsm, cudaDevAttrMultiProcessorCount, dev);
        // whole-level half-sweeps by default: with two z planes per half-sweep thread the y-slab wavefront
        // (ia_poisson_slab_rows) no longer shortens the step
        mg->slab_rows = 0;
    }
    return IA_OK;
}

void mg_destroy(ia_handle* h) {
    PoissonMG* mg = h->mg;
    if (!mg) return;
    for (int l = 0; l < MG_MAX_LEVELS; ++l) {
        MGLevel& L = mg->lev[l];
        cudaFree(L.x); cudaFree(L.b); cudaFree(L.r); cudaFree(L.L); cudaFree(L.iD);
        cudaFree(L.x32); cudaFree(L.b32); cudaFree(L.r32); cudaFree(L.L32); cudaFree(L.iD32); cudaFree(L.L16);
    }
    cudaFree(mg->r); cudaFree(mg->s); cudaFree(mg->p); cudaFree(mg->q);
    cudaFree(mg->p32); cudaFree(mg->q32); cudaFree(mg->e32);
    cudaFree(mg->rl32); cudaFree(mg->nl32); cudaFree(mg->t32);
    cudaFree(mg->partial); cudaFree(mg->dsc); cudaFree(mg->fcg); cudaFree(mg->diag64);
    for (int k = 0; k < 2; ++k)
        if (mg->vgraph[k]) cudaGraphExecDestroy(mg->vgraph[k]);
    if (mg->capture) cudaStreamDestroy(mg->capture);
    if (mg->hsc) cudaFreeHost(mg->hsc);
    delete mg;
    h->mg = nullptr;
}

// build every level's operator from the fine coefficients L0 (μ₀, FP64)
static cudaError_t mg_setup(ia_handle* h, const double* L0) {
    PoissonMG* mg = h->mg;
    cudaStream_t st = h->stream;
    const bool mixed = h->cfg.poisson_mode != IA_POISSON_FP64;
    MGLevel& F = mg->lev[0];
    const long long nv = F.g.N * F.g.D;
    if (!mixed) { set_diag64_k<<<mg->kb, KTHREADS, 0, st>>>(F.g, L0, mg->diag64); ia::note_launch(); }
    if (!mixed) {
        cudaMemcpyAsync(F.L, L0, 8 * nv, cudaMemcpyDeviceToDevice, st);
        { set_diag_k<double><<<grd(F.g), blk(), 0, st>>>(F.g, F.L, F.iD); ia::note_launch(); }
        for (int l = 1; l < mg->nlev; ++l) {
            { restrict_L_k<double><<<grd(mg->lev[l].g), blk(), 0, st>>>(mg->lev[l].g, mg->lev[l - 1].g,
                                                                       mg->lev[l - 1].L, mg->lev[l].L); ia::note_launch(); }
            { set_diag_k<double><<<grd(mg->lev[l].g), blk(), 0, st>>>(mg->lev[l].g, mg->lev[l].L, mg->lev[l].iD); ia::note_launch(); }
        }
    } else {
        // FP64 diagonal, FP32 (and FP16) coefficient copies and the FP32 inverse diagonal in one pass
        const dim3 gg((F.g.n[0] + 31) / 32, (F.g.n[1] + 7) / 8, F.g.D == 3 ? F.g.n[2] : 1);
        __half* l16 = mg->coef16 ? F.L16 : nullptr;
        LAUNCH_D(F.g, setup_fine_k, gg, blk(), F.g, L0, mg->diag64, F.L32, l16, F.iD32);
        for (int l = 1; l < mg->nlev; ++l) {
            { restrict_L_k<float><<<grd(mg->lev[l].g), blk(), 0, st>>>(mg->lev[l].g, mg->lev[l - 1].g,
                                                                      mg->lev[l - 1].L32, mg->lev[l].L32); ia::note_launch(); }
            { set_diag_k<float><<<grd(mg->lev[l].g), blk(), 0, st>>>(mg->lev[l].g, mg->lev[l].L32, mg->lev[l].iD32); ia::note_launch(); }
        }
    }
    return cudaGetLastError();
}

// s = M r (one V-cycle)
static cudaError_t mg_precondition(ia_handle* h) {
    PoissonMG* mg = h->mg;
    cudaStream_t st = h->stream;
    MGLevel& F = mg->lev[0];
    const long long N = F.g.N;
    cudaError_t e;
    if (h->cfg.poisson_mode != IA_POISSON_FP64) {
        int tk = timing_begin(h, TK_MG_TRANSFER);
        { to_f32_k<<<1216, 256, 0, st>>>(N, mg->r, F.b32); ia::note_launch(); }
        timing_end(h, tk);
        tk = timing_begin(h, TK_MG_SMOOTH);
        e = vcycle_run<float>(h, mg, st);
        timing_end(h, tk);
        if (e != cudaSuccess) return e;
        { to_f64_k<<<1216, 256, 0, st>>>(N, F.x32, mg->s); ia::note_launch(); }
    } else {
        cudaMemcpyAsync(F.b, mg->r, 8 * N, cudaMemcpyDeviceToDevice, st);
        int tk = timing_begin(h, TK_MG_SMOOTH);
        e = vcycle_run<double>(h, mg, st);
        timing_end(h, tk);
        if (e != cudaSuccess) return e;
        cudaMemcpyAsync(mg->s, F.x, 8 * N, cudaMemcpyDeviceToDevice, st);
    }
    return cudaGetLastError();
}

// r = z - A x with the FP64 operator and the precomputed diagonal; L∞(r), as the bit pattern of |r|,
// into *dlinf
static void true_residual(PoissonMG* mg, const Grid& g, const double* L, const double* zz, const double* xv,
                          unsigned long long* dlinf, cudaStream_t st, float* r32 = nullptr, float* e32 = nullptr) {
    unsigned long long* pmax = reinterpret_cast<unsigned long long*>(mg->partial);
    LAUNCH_D(g, true_resid_tile_k, mv_tile_grid(g), KTHREADS, g, L, mg->diag64, zz, xv, mg->r, pmax, r32, e32);
    { finalize_max_k<<<1, 1024, 0, st>>>(pmax, mg->mvb, dlinf); ia::note_launch(); }
}

static double read_linf(ia_handle* h, unsigned long long* dlinf) {
    unsigned long long v = 0;
    cudaMemcpyAsync(&h->mg->hsc[0], dlinf, 8, cudaMemcpyDeviceToHost, h->stream);
    cudaStreamSynchronize(h->stream);
    std::memcpy(&v, &h->mg->hsc[0], 8);
    double d;
    std::memcpy(&d, &v, 8);
    return d;
}

// Mixed precision: FP64 defect correction x += e, e from an inner flexible CG run
// entirely in FP32 (operator, preconditioner, vectors) on A e = r, started from the FP64
// true residual; inner dot products are block sums in FP32 reduced across blocks in
// FP64 and the CG scalars are FP64.  The inner preconditioner is the FP32 V-cycle
// (IA_POISSON_MIXED) or, for IA_POISSON_LEARNED, the mode set by ia_poisson_precond.
static int poisson_solve_mixed(ia_handle* h, double* xv, const double* zz, const double* L, double tol, int itmx,
                               int* iters, double* resid) {
    PoissonMG* mg = h->mg;
    cudaStream_t st = h->stream;
    const Grid& g = h->g;
    const dim3 gb = grd(g);
    MGLevel& F = mg->lev[0];
    const long long N = g.N;
    unsigned long long* dlinf = reinterpret_cast<unsigned long long*>(mg->dsc + 8);
    double* hdots = mg->dsc + 12;                                  // hybrid n·t, n·An
    const bool learned = h->cfg.poisson_mode == IA_POISSON_LEARNED;
    // inner residual: the V-cycle reads its right-hand side from F.b32, so the plain mixed
    // mode keeps the residual there; the learned modes keep it apart
    float* rr = learned ? mg->rl32 : F.b32;
    int mode = learned ? mg->precond : IA_PRECOND_VCYCLE;
    auto vcyc = [&]() -> cudaError_t {
        const int tk = timing_begin(h, TK_MG_SMOOTH);
        const cudaError_t e = vcycle_run<float>(h, mg, st);
        timing_end(h, tk);
        mg->stats[1]++;
        return e;
    };
    auto net = [&](const float* in) -> bool {
        const int tk = timing_begin(h, TK_NN);
        const int rc = nn_apply(h, in, F.L32, mg->nl32, g.n[0] - 2, g.n[1] - 2, g.n[2] - 2, N);
        timing_end(h, tk);
        mg->stats[0]++;
        return rc == IA_OK;
    };
    // sv ≈ A⁻¹ rr
    auto precond = [&](float*& sv) -> bool {
        if (mode == IA_PRECOND_NONE) {
            sv = rr;
            return true;
        }
        if (mode == IA_PRECOND_NET) {
            sv = mg->nl32;
            return net(rr);
        }
        if (rr != F.b32) cudaMemcpyAsync(F.b32, rr, 4 * N, cudaMemcpyDeviceToDevice, st);
        sv = F.x32;
        if (vcyc() != cudaSuccess) return false;
        if (mode != IA_PRECOND_HYBRID) return true;
        // hybrid: the net corrects what the V-cycle left, s += ω net(t) with t = r - A s and
        // ω = (n·t)/(n·An), the energy-optimal step along n = net(t)
        int tk = timing_begin(h, TK_KRYLOV);
        if (g.D == 3) { residual_k<float, 3><<<cell_grid(g), blk(), 0, st>>>(g, F.L32, rr, F.x32, mg->t32); ia::note_launch(); }
        else { residual_k<float, 2><<<cell_grid(g), blk(), 0, st>>>(g, F.L32, rr, F.x32, mg->t32); ia::note_launch(); }
        timing_end(h, tk);
        if (!net(mg->t32)) return false;
        tk = timing_begin(h, TK_KRYLOV);
        LAUNCH_D(g, energy_dots_k, mg->kb, KTHREADS, g, F.L32, mg->nl32, mg->t32, mg->partial);
        { finalize_k<<<1, 1024, 0, st>>>(mg->partial, mg->kb, 2, hdots); ia::note_launch(); }
        { add_scaled_k<<<mg->kb, KTHREADS, 0, st>>>(g, hdots, mg->nl32, F.x32); ia::note_launch(); }
        timing_end(h, tk);
        return cudaGetLastError() == cudaSuccess;
    };
    int total = 0;
    int tk = timing_begin(h, TK_KRYLOV);
    // every FP64 residual also starts the next inner solve: rr = float(r), e32 = 0
    true_residual(mg, g, L, zz, xv, dlinf, st, rr, mg->e32);
    timing_end(h, tk);
    double res = read_linf(h, dlinf);
    while (!(res <= tol) && total < itmx) {
        const double target = std::fmax(0.5 * tol / res, mg->inner_rtol) * res;
        FcgDev* S = mg->fcg;
        // the reductions' last-block counters start from zero in every inner solve (each launch leaves
        // them at zero, but not one that an error cut short)
        cudaMemsetAsync(&S->done_dot, 0, 2 * sizeof(unsigned int), st);
        for (int it = 0; it < mg->inner_max && total < itmx; ++it) {
            float* sv = nullptr;
            if (!precond(sv)) return IA_ERR_CUDA;
            // β, the direction, q = A p, α and the update without a host round trip; one read-back of
            // the inner residual and the breakdown flag per step
            tk = timing_begin(h, TK_KRYLOV);
            { dot2_32_k<<<mg->kb, KTHREADS, 0, st>>>(N, sv, mg->q32, rr, mg->partial, S, it == 0 ? 1 : 0); ia::note_launch(); }
            { xpby32_k<<<mg->kb, KTHREADS, 0, st>>>(N, sv, S, mg->p32); ia::note_launch(); }
            LAUNCH_D(g, matvec32_tile_k, mv_tile_grid(g), KTHREADS, g, F.L32, mg->p32, mg->q32, mg->partial, S);
            { update32_k<<<mg->kb, KTHREADS, 0, st>>>(N, S, mg->p32, mg->q32, mg->e32, rr); ia::note_launch(); }
            timing_end(h, tk);
            cudaMemcpyAsync(mg->hsc + 2, &S->rin, 8, cudaMemcpyDeviceToHost, st);
            if (cudaStreamSynchronize(st) != cudaSuccess) return IA_ERR_CUDA;
            unsigned int rin_bits = 0;
            int stop = 0;
            std::memcpy(&rin_bits, reinterpret_cast<const char*>(mg->hsc + 2), 4);
            std::memcpy(&stop, reinterpret_cast<const char*>(mg->hsc + 2) + 4, 4);
            ++total;
            mg->stats[3]++;
            if (stop) break;
            float rinf;
            std::memcpy(&rinf, &rin_bits, 4);
            if (double(rinf) <= target) break;
        }
        tk = timing_begin(h, TK_KRYLOV);
        LAUNCH_D(g, add_correction_k, mv_tile_grid(g), KTHREADS, g, mg->e32, xv);
        true_residual(mg, g, L, zz, xv, dlinf, st, rr, mg->e32);
        timing_end(h, tk);
        const double res_old = res;
        res = read_linf(h, dlinf);
        mg->stats[4]++;
        // fallback: a correction that fails to halve the FP64 true residual (or a net
        // kernel that reported a timeout) hands the rest of the solve to the V-cycle
        if (learned && mode != IA_PRECOND_VCYCLE && (!(res <= 0.5 * res_old) || nn_error_flag(h))) {
            mode = IA_PRECOND_VCYCLE;
            mg->stats[2]++;
        }
    }
    { perbc_k<<<unsigned((bc_plane_cells(g) + 255) / 256), 256, 0, st>>>(g, xv); ia::note_launch(); }
    if (cudaGetLastError() != cudaSuccess) return IA_ERR_CUDA;
    *iters = total;
    *resid = res;
    return (res <= tol) ? IA_OK : IA_WARN_NOT_CONVERGED;
}

// r = z - A x over interior cells; L∞(r) to the host
int poisson_residual(ia_handle* h, double* r, const double* x, const double* z, const double* L, double* linf) {
    cudaStream_t st = h->stream;
    unsigned long long* d = reinterpret_cast<unsigned long long*>(h->dscalar + 60);
    cudaMemsetAsync(d, 0, 8, st);
    LAUNCH_D(h->g, true_resid_k, kblocks(h->g), KTHREADS, h->g, L, nullptr, z, x, r, d);
    unsigned long long v = 0;
    cudaMemcpyAsync(&v, d, 8, cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return IA_ERR_CUDA;
    if (linf) std::memcpy(linf, &v, 8);
    return IA_OK;
}

// Solve A x = z to L∞(z - A x) <= tol (x holds the initial guess); L = μ₀.
int poisson_solve(ia_handle* h, double* xv, const double* zz, const double* L, double tol, int itmx, int* iters,
                  double* resid) {
    PoissonMG* mg = h->mg;
    if (!mg) return IA_ERR_INVALID;
    if (h->cfg.poisson_mode != IA_POISSON_FP64) {
        if (mg_setup(h, L) != cudaSuccess) return IA_ERR_CUDA;
        return poisson_solve_mixed(h, xv, zz, L, tol, itmx, iters, resid);
    }
    cudaStream_t st = h->stream;
    const Grid& g = h->g;
    const dim3 gb = grd(g);
    if (mg_setup(h, L) != cudaSuccess) return IA_ERR_CUDA;
    unsigned long long* dlinf = reinterpret_cast<unsigned long long*>(mg->dsc + 8);
    double* dots = mg->dsc;
    int tk = timing_begin(h, TK_KRYLOV);
    true_residual(mg, g, L, zz, xv, dlinf, st);
    timing_end(h, tk);
    double res = read_linf(h, dlinf);
    int it = 0;
    double rho_prev = 0.0, alpha_prev = 0.0;
    while (!(res <= tol) && it < itmx) {
        if (mg_precondition(h) != cudaSuccess) return IA_ERR_CUDA;
        tk = timing_begin(h, TK_KRYLOV);
        { dot2_k<<<mg->kb, KTHREADS, 0, st>>>(g, mg->s, mg->q, mg->r, mg->partial); ia::note_launch(); }
        { finalize_k<<<1, 1024, 0, st>>>(mg->partial, mg->kb, 2, dots); ia::note_launch(); }
        timing_end(h, tk);
        cudaMemcpyAsync(mg->hsc + 2, dots, 16, cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) return IA_ERR_CUDA;
        const double sq = mg->hsc[2], sr = mg->hsc[3];
        // flexible CG: β = s_k·(r_k - r_{k-1}) / (s_{k-1}·r_{k-1}) with r_k - r_{k-1} = -α q_{k-1}
        const double beta = (it == 0) ? 0.0 : (-alpha_prev * sq) / rho_prev;
        const double rho = sr;
        tk = timing_begin(h, TK_KRYLOV);
        { xpby_k<<<mg->kb, KTHREADS, 0, st>>>(g, mg->s, beta, mg->p); ia::note_launch(); }
        LAUNCH_D(g, matvec_dot_k, mg->kb, KTHREADS, g, L, mg->diag64, mg->p, mg->q, mg->partial);
        { finalize_k<<<1, 1024, 0, st>>>(mg->partial, mg->kb, 1, dots); ia::note_launch(); }
        timing_end(h, tk);
        cudaMemcpyAsync(mg->hsc + 2, dots, 8, cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) return IA_ERR_CUDA;
        const double pq = mg->hsc[2];
        if (!(pq != 0.0) || !std::isfinite(pq)) break;
        const double alpha = rho / pq;
        cudaMemsetAsync(dlinf, 0, 8, st);
        tk = timing_begin(h, TK_KRYLOV);
        { update_k<<<mg->kb, KTHREADS, 0, st>>>(g, alpha, mg->p, mg->q, xv, mg->r, dlinf); ia::note_launch(); }
        timing_end(h, tk);
        res = read_linf(h, dlinf);
        rho_prev = rho;
        alpha_prev = alpha;
        ++it;
    }
    { perbc_k<<<unsigned((bc_plane_cells(g) + 255) / 256), 256, 0, st>>>(g, xv); ia::note_launch(); }
    if (cudaGetLastError() != cudaSuccess) return IA_ERR_CUDA;
    *iters = it;
    *resid = res;
    return (res <= tol) ? IA_OK : IA_WARN_NOT_CONVERGED;
}

}  // namespace ia
