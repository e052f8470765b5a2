// Ghost-cell rules evaluated on the fly.
//
// The reference applies its boundary conditions as slice copies over
// j = 1..D (low face, then high face).  Because every copy reads from a
// position whose other coordinates were already fixed, the final value of any
// ghost equals the value at a source position obtained by mapping each
// boundary coordinate independently.  The functions below return that source
// (or a Dirichlet value) so kernels read ghosts without a separate pass.
#pragma once
#include "ia_core.cuh"

namespace ia {

// WaterLily BC!(a, A, false, perdir) for component i at coordinate c:
// the normal component is A[i] on the low ghost, the low wall face and the high
// wall face of a non-periodic dimension i; other coordinates copy the adjacent
// interior cell (zero gradient) or wrap (periodic).  Returns true when the value
// is the Dirichlet constant; otherwise c becomes the source coordinate.
__device__ __forceinline__ bool vel_bc(const Grid& g, int i, int c[3]) {
    if (!g.isper(i) && (c[i] == 0 || c[i] == 1 || c[i] == g.n[i] - 1)) return true;
    for (int e = 0; e < g.D; ++e) c[e] = bc_src(g, e, c[e]);
    return false;
}

// BCv! / BCv1D! / BCf!(d, ·) for a d-face field (src/VOFutil.jl:76-119):
// along a non-periodic d the low ghost copies index 2 and the high ghost
// (the upper boundary face itself) keeps its own value; every other
// dimension is zero-gradient or periodic.  Returns true when the position is
// that never-written upper face (c then holds it unchanged).
__device__ __forceinline__ bool face_bc(const Grid& g, int d, int c[3]) {
    bool upper = false;
    for (int e = 0; e < g.D; ++e) {
        const int L = g.n[e] - 1;
        if (g.isper(e)) {
            c[e] = bc_src(g, e, c[e]);
        } else if (e == d) {
            if (c[e] == 0) c[e] = 2;
            else if (c[e] == L) upper = true;
        } else {
            c[e] = bc_src(g, e, c[e]);
        }
    }
    return upper;
}

// The cells BC! changes: the planes c[e] in {0, 1, n_e - 1} of each dimension (ghost layers and
// Dirichlet wall faces), numbered dimension by dimension, plane by plane, x fastest within a plane.
// bc_plane_cells() counts them; bc_plane_cell() gives the coordinates of number t (false when t is
// past the end).  Cells on an edge or corner appear once per plane they lie on.
__host__ __device__ inline long long bc_plane_cells(const Grid& g) {
    const long long n0 = g.n[0], n1 = g.n[1], n2 = g.n[2];
    return 3 * n1 * n2 + 3 * n0 * n2 + (g.D == 3 ? 3 * n0 * n1 : 0);
}
__host__ __device__ inline int bc_plane_coord(int which, int n) { return which == 0 ? 0 : (which == 1 ? 1 : n - 1); }
__host__ __device__ inline bool bc_plane_cell(const Grid& g, long long t, int c[3]) {
    const long long n0 = g.n[0], n1 = g.n[1], n2 = g.n[2];
    const long long a0 = n1 * n2, a1 = n0 * n2, a2 = n0 * n1;   // cells per plane of dimension 0, 1, 2
    if (t < 3 * a0) {
        const long long r = t % a0;
        c[0] = bc_plane_coord(int(t / a0), g.n[0]);
        c[1] = int(r % n1);
        c[2] = int(r / n1);
        return true;
    }
    t -= 3 * a0;
    if (t < 3 * a1) {
        const long long r = t % a1;
        c[1] = bc_plane_coord(int(t / a1), g.n[1]);
        c[0] = int(r % n0);
        c[2] = int(r / n0);
        return true;
    }
    t -= 3 * a1;
    if (g.D == 3 && t < 3 * a2) {
        const long long r = t % a2;
        c[2] = bc_plane_coord(int(t / a2), g.n[2]);
        c[0] = int(r % n0);
        c[1] = int(r / n0);
        return true;
    }
    return false;
}

__device__ __forceinline__ bool is_interior(const Grid& g, const int c[3]) {
    for (int e = 0; e < g.D; ++e)
        if (c[e] < 1 || c[e] > g.n[e] - 2) return false;
    return true;
}

__device__ __forceinline__ void coords3(const Grid& g, long long O, int c[3]) {
    c[0] = int(O % g.n[0]);
    const long long r = O / g.n[0];
    c[1] = int(r % g.n[1]);
    c[2] = int(r / g.n[1]);
}

__device__ __forceinline__ long long lin3(const Grid& g, const int c[3]) { return lin(g, c[0], c[1], c[2]); }

constexpr unsigned long long kOneBits = 0x3FF0000000000000ull;
constexpr unsigned long long kAbsMask = 0x7FFFFFFFFFFFFFFFull;
__device__ __forceinline__ unsigned long long dbits(double v) { return (unsigned long long)__double_as_longlong(v); }

// Monotone integer key of a double (total order on non-NaN values) for
// comparisons, min and max without FP64 instructions.
__device__ __forceinline__ long long okey(double v) {
    const long long b = __double_as_longlong(v);
    return b ^ (long long)((unsigned long long)(b >> 63) >> 1);
}
__device__ __forceinline__ double dmin(double a, double b) { return okey(b) < okey(a) ? b : a; }
__device__ __forceinline__ double dmax(double a, double b) { return okey(a) < okey(b) ? b : a; }
__device__ __forceinline__ bool dlt(double a, double b) { return okey(a) < okey(b); }
__device__ __forceinline__ double dabs(double v) { return __longlong_as_double(__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFll); }

// Density at the lower d-face from two cell fractions: λρ + (1-λρ)(fa+fb)/2
// (getρ(d,I,f,λρ), src/VOFutil.jl:176).  Full/empty pairs skip the FP64 work.
struct RhoFace {
    double lrho, one_m, rho1;   // λρ, 1-λρ, λρ + (1-λρ)·1
    __device__ __forceinline__ double operator()(double fa, double fb) const {
        const unsigned long long a = dbits(fa), b = dbits(fb);
        if (a == b && a == 0ull) return lrho;
        if (a == b && a == kOneBits) return rho1;
        return lrho + one_m * ((fa + fb) / 2.0);
    }
};

}  // namespace ia
