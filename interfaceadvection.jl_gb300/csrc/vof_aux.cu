// Initialisation and unit-parity kernels around the VOF sweep:
// applyVOF! (src/VOFutil.jl:9-37), reconstructInterface! + BCVOF!
// (src/normalEstimation.jl:10-28, src/VOFutil.jl:44-62), getVOFFlux! with
// caller-supplied α/n̂ (src/advection.jl:108-137), BCf! ghosts and a
// deterministic interior sum used for mass diagnostics.
#include <cuda_runtime.h>

#include "ia_bc.cuh"
#include "ia_geom.cuh"
#include "vof.cuh"

namespace ia {

namespace {

__device__ __forceinline__ bool interior(const Grid& g, int x, int y, int z) {
    if (x < 1 || x > g.n[0] - 2 || y < 1 || y > g.n[1] - 2) return false;
    if (g.D == 3 && (z < 1 || z > g.n[2] - 2)) return false;
    return true;
}

template <int D>
__global__ void apply_vof_k(Grid g, const double* __restrict__ sdf, double* f, double* alpha, double* nhat) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y, z = blockIdx.z;
    if (x >= g.n[0] || y >= g.n[1] || !interior(g, x, y, z)) return;
    const long long I = lin(g, x, y, z);
    double n[3] = {0.0, 0.0, 0.0}, sn = 0.0, sn2 = 0.0;
#pragma unroll
    for (int i = 0; i < D; ++i) {
        const double dd = sdf[(1 + 2 * i) * g.N + I] - sdf[(2 + 2 * i) * g.N + I];
        n[i] = dd;
        nhat[i * g.N + I] = dd;
        sn += dd;
        sn2 += dd * dd;
    }
    const double a = sn / 2.0 - sqrt(sn2) * sdf[I];
    alpha[I] = a;
    double v = get_volume_fraction<D>(n, a);
    const double tol = 10.0 * 2.220446049250313e-16;
    f[I] = (v < tol) ? 0.0 : ((v > 1.0 - tol) ? 1.0 : v);
}

// one thread per cell of the boundary planes (bc_plane_cell); the interior cells among them return
__global__ void ghosts_k(Grid g, double* f) {
    int cc[3];
    if (!bc_plane_cell(g, blockIdx.x * (long long)blockDim.x + threadIdx.x, cc)) return;
    const int x = cc[0], y = cc[1], z = cc[2];
    if (interior(g, x, y, z)) return;
    const int sz = g.D == 3 ? bc_src(g, 2, z) : 0;
    f[lin(g, x, y, z)] = f[lin(g, bc_src(g, 0, x), bc_src(g, 1, y), sz)];
}

template <int D>
__global__ void reconstruct_k(Grid g, int scheme, const double* __restrict__ f, double* alpha, double* nhat) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y, z = blockIdx.z;
    if (x >= g.n[0] || y >= g.n[1] || !interior(g, x, y, z)) return;
    const long long I = lin(g, x, y, z);
    const double fc = f[I];
    double n[3] = {0.0, 0.0, 0.0}, a = 0.0;
    if (!(fc == 0.0 || fc == 1.0)) {
        Stencil S;
        S.f = f;
        S.c = I;
        S.s[0] = g.s[0];
        S.s[1] = g.s[1];
        S.s[2] = g.s[2];
        interface_normal<D>(scheme, S, n);
        a = get_intercept<D>(n, fc);
    }
    for (int i = 0; i < D; ++i) nhat[i * g.N + I] = n[i];
    alpha[I] = a;
}

// BCVOF! ghosts: f from the full boundary map; α, n̂ copied only along
// periodic dimensions (zero-gradient sides leave them untouched).
__global__ void bcvof_ghosts_k(Grid g, double* f, double* alpha, double* nhat) {
    int cc[3];
    if (!bc_plane_cell(g, blockIdx.x * (long long)blockDim.x + threadIdx.x, cc)) return;
    const int x = cc[0], y = cc[1], z = cc[2];
    if (interior(g, x, y, z)) return;
    const long long O = lin(g, x, y, z);
    const int sz = g.D == 3 ? bc_src(g, 2, z) : 0;
    f[O] = f[lin(g, bc_src(g, 0, x), bc_src(g, 1, y), sz)];
    int c[3] = {x, y, z};
    for (int e = 0; e < g.D; ++e)
        if (g.isper(e) && (c[e] == 0 || c[e] == g.n[e] - 1)) c[e] = bc_src(g, e, c[e]);
    const long long P = lin(g, c[0], c[1], c[2]);
    if (P == O) return;
    alpha[O] = alpha[P];
    for (int i = 0; i < g.D; ++i) nhat[i * g.N + O] = nhat[i * g.N + P];
}

template <int D>
__global__ void vof_flux_k(Grid g, double* fF, const double* __restrict__ f, const double* __restrict__ alpha,
                           const double* __restrict__ nhat, const double* __restrict__ u,
                           const double* __restrict__ u0, double dt, int d, double* rhouf, double lrho) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y, z = blockIdx.z;
    if (x >= g.n[0] || y >= g.n[1]) return;
    const long long K = lin(g, x, y, z);
    const int c[3] = {x, y, z};
    bool face = true;
    for (int e = 0; e < D; ++e) {
        const int hi = (e == d) ? g.n[e] - 1 : g.n[e] - 2;
        if (c[e] < 1 || c[e] > hi) face = false;
    }
    double F = 0.0;
    if (face) {
        const double dl = dt / 2.0 * (u[d * g.N + K] + u0[d * g.N + K]);
        if (dl != 0.0) {
            const long long C = dl > 0.0 ? K - g.s[d] : K;
            double sa = 0.0;
            for (int i = 0; i < D; ++i) sa += fabs(nhat[i * g.N + C]);
            const double fC = f[C];
            if (sa == 0.0 || fC == 0.0 || fC == 1.0) {
                F = fC * dl;
            } else {
                const double b = dl > 0.0 ? alpha[C] - nhat[d * g.N + C] * (1.0 - dl) : alpha[C];
                double n[3] = {0.0, 0.0, 0.0};
                for (int i = 0; i < D; ++i) n[i] = nhat[i * g.N + C] * (i == d ? fabs(dl) : 1.0);
                F = get_volume_fraction<D>(n, b) * dl;
            }
            if (rhouf) rhouf[d * g.N + K] += dl * lrho + (1.0 - lrho) * F;
        }
    }
    fF[K] = F;
}

__global__ void sum_rows_k(Grid g, const double* __restrict__ f, double* partial) {
    __shared__ double red[256];
    const long long rows = (long long)(g.n[1] - 2) * (g.D == 3 ? (g.n[2] - 2) : 1);
    double acc = 0.0;
    for (long long r = blockIdx.x; r < rows; r += gridDim.x) {
        const int y = 1 + int(r % (g.n[1] - 2));
        const int z = (g.D == 3) ? 1 + int(r / (g.n[1] - 2)) : 0;
        const double* row = f + lin(g, 0, y, z);
        for (int x = 1 + threadIdx.x; x <= g.n[0] - 2; x += blockDim.x) acc += row[x];
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

__global__ void sum_partials_k(const double* partial, int n, double* out) {
    __shared__ double red[1024];
    double acc = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) acc += partial[i];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0];
}

inline dim3 blk3() { return dim3(32, 8, 1); }
inline dim3 grd3(const Grid& g) { return dim3((g.n[0] + 31) / 32, (g.n[1] + 7) / 8, g.n[2]); }

}  // namespace

cudaError_t fill_ghosts_scalar(const Grid& g, double* f, cudaStream_t st) {
    { ghosts_k<<<unsigned((bc_plane_cells(g) + 255) / 256), 256, 0, st>>>(g, f); ia::note_launch(); }
    return cudaGetLastError();
}

cudaError_t apply_vof(const Grid& g, const double* sdf, double* f, double* alpha, double* nhat, cudaStream_t st) {
    if (g.D == 2) { apply_vof_k<2><<<grd3(g), blk3(), 0, st>>>(g, sdf, f, alpha, nhat); ia::note_launch(); }
    else { apply_vof_k<3><<<grd3(g), blk3(), 0, st>>>(g, sdf, f, alpha, nhat); ia::note_launch(); }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return fill_ghosts_scalar(g, f, st);
}

cudaError_t reconstruct(const Grid& g, int scheme, double* f, double* alpha, double* nhat, cudaStream_t st) {
    if (g.D == 2) { reconstruct_k<2><<<grd3(g), blk3(), 0, st>>>(g, scheme, f, alpha, nhat); ia::note_launch(); }
    else { reconstruct_k<3><<<grd3(g), blk3(), 0, st>>>(g, scheme, f, alpha, nhat); ia::note_launch(); }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    { bcvof_ghosts_k<<<unsigned((bc_plane_cells(g) + 255) / 256), 256, 0, st>>>(g, f, alpha, nhat); ia::note_launch(); }
    return cudaGetLastError();
}

cudaError_t vof_flux(const Grid& g, double* fF, const double* f, const double* alpha, const double* nhat,
                     const double* u, const double* u0, double dt, int d, double* rhouf, double lrho,
                     cudaStream_t st) {
    if (g.D == 2) { vof_flux_k<2><<<grd3(g), blk3(), 0, st>>>(g, fF, f, alpha, nhat, u, u0, dt, d, rhouf, lrho); ia::note_launch(); }
    else { vof_flux_k<3><<<grd3(g), blk3(), 0, st>>>(g, fF, f, alpha, nhat, u, u0, dt, d, rhouf, lrho); ia::note_launch(); }
    return cudaGetLastError();
}

cudaError_t interior_sum(const Grid& g, const double* f, double* partial, double* out, cudaStream_t st) {
    const int nb = 1024;
    { sum_rows_k<<<nb, 256, 0, st>>>(g, f, partial); ia::note_launch(); }
    { sum_partials_k<<<1, 1024, 0, st>>>(partial, nb, out); ia::note_launch(); }
    return cudaGetLastError();
}

}  // namespace ia
