// Core device-side definitions shared by every kernel of libintfadv_gb300.
//
// Memory layout (the reference's Julia layout, so Julia CuArrays can be passed
// straight through the C-ABI): column-major, x fastest, one ghost layer on each
// side (Ng = N + 2), vector fields SoA with the component index last
// (component d of cell I lives at I + d * total).  Coordinates are 0-based:
// ghost 0, interior 1..Ng-2, ghost Ng-1.  A vector entry u[I, d] sits on the
// lower d-face of cell I (WaterLily's staggered arrangement).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/intfadv.h"

namespace ia {

struct Grid {
    int D;          // 2 or 3
    int per;        // bit j set <=> dimension j periodic
    int n[3];       // ghost-inclusive sizes (n[2] == 1 in 2D)
    long long s[3]; // strides (1, n0, n0*n1)
    long long N;    // cells per scalar field

    __host__ __device__ bool isper(int d) const { return (per >> d) & 1; }
};

inline Grid make_grid(int D, int per, const int64_t Nint[3]) {
    Grid g;
    g.D = D;
    g.per = per;
    for (int d = 0; d < 3; ++d) g.n[d] = (d < D) ? int(Nint[d] + 2) : 1;
    g.s[0] = 1;
    g.s[1] = g.n[0];
    g.s[2] = (long long)g.n[0] * g.n[1];
    g.N = (long long)g.n[0] * g.n[1] * g.n[2];
    return g;
}

// Boundary-condition source coordinate of a (possibly ghost) coordinate along
// dimension e: zero-gradient copies the adjacent interior cell, periodic wraps.
// Composing this per dimension reproduces BCf! / BCVOF!'s f part
// (src/VOFutil.jl:44-75), whose slice loops over j = 1..D make every ghost,
// corners included, equal to the interior cell reached by mapping each
// out-of-range coordinate independently.
__device__ __forceinline__ int bc_src(const Grid& g, int e, int c) {
    const int L = g.n[e] - 1;
    if (c == 0) return g.isper(e) ? L - 1 : 1;
    if (c == L) return g.isper(e) ? 1 : L - 1;
    return c;
}

__device__ __forceinline__ long long lin(const Grid& g, int x, int y, int z) {
    return x + g.s[1] * y + g.s[2] * z;
}

// Host-side count of kernel launches issued by this library (every launch site
// calls note_launch after issuing its kernel).
void note_launch();
void note_launches(long long n);   // kernels of a graph launch (or, negative, of a capture)
long long launch_count();

// Order-preserving map of a double onto uint64 (for atomicMax / atomicMin).
__device__ __forceinline__ unsigned long long ord_enc(double v) {
    unsigned long long b = __double_as_longlong(v);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__host__ __device__ inline double ord_dec(unsigned long long e) {
    unsigned long long b = (e >> 63) ? (e & 0x7FFFFFFFFFFFFFFFull) : ~e;
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)b);
#else
    double v;
    __builtin_memcpy(&v, &b, 8);
    return v;
#endif
}

// Device-side fill/error status of one call (reportFillError, src/advection.jl:145-189).
struct DevStatus {
    unsigned int flags;                 // IA_FLAG_* bits
    unsigned int dir;                   // last sweep direction that flagged
    unsigned long long max_enc;         // ord_enc of the largest fraction seen past tol
    unsigned long long min_enc;         // ord_enc of the smallest
    unsigned long long max_key;         // (float bits of over-fill) << 32 | cell
    unsigned long long min_key;         // (float bits of under-fill) << 32 | cell
    unsigned int list_count[32];        // compaction counters (two per sweep)
    double scratch[8];                  // reductions (CFL, norms)
};

}  // namespace ia
