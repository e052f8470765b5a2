// Level-set reinitialisation of src/redistaning.jl: ϕ = 2f - 1 (LevelSet, :13-25), the
// pseudo-time right-hand side L = ϕ_ini (1 - |∇ϕ|) with second-order ENO one-sided
// derivatives (computeL!, :64-83; ∇ϕᵢ², :118-143; the Neumann and periodic boundary
// building blocks :86-110), and the three-stage SSP Runge-Kutta march (redistaning!,
// :42-54; _redistaningStage!, :27-30) with BCf! ghosts after every stage.
//
// One kernel computes L over all interior cells and all directions (the reference's
// per-direction lower / inner / upper loops fused, same per-direction sum order); one
// kernel applies the stage update; the scalar ghost kernel of the VOF module applies BCf!.
#include <cuda_runtime.h>

#include <cmath>

#include "capi_internal.cuh"
#include "ia_bc.cuh"

namespace ia {
namespace {

inline dim3 blk() { return dim3(32, 8, 1); }
inline dim3 grd(const Grid& g) { return dim3((g.n[0] + 31) / 32, (g.n[1] + 7) / 8, g.n[2]); }

__device__ __forceinline__ double minmod(double a, double b) { return fabs(a) <= fabs(b) ? a : b; }

// ∇ϕᵢ²(a,b,c,d,e,s): ENO2 (minmod-limited) one-sided derivatives, upwinded by s
__device__ __forceinline__ double grad2(double a, double b, double c, double d, double e, double s) {
    const double dp = d - c, dm = c - b;
    const double d2p = e + c - 2.0 * d, d2o = d + b - 2.0 * c, d2m = c + a - 2.0 * b;
    const double dR = dp - minmod(d2p, d2o) / 2.0;
    const double dL = dm + minmod(d2o, d2m) / 2.0;
    const double wR = dR * s, wL = dL * s;
    if (wR < 0.0 && (wR + wL) < 0.0) return dR * dR;
    if (wL > 0.0 && (wR + wL) > 0.0) return dL * dL;
    return 0.0;
}

__device__ __forceinline__ double sgn(double v) { return v > 0.0 ? 1.0 : (v < 0.0 ? -1.0 : v); }

// L[I] = ϕini[I] (1 - sqrt(Σ_i ∇ϕᵢ²)) on interior cells
__global__ void computeL_k(Grid g, const double* __restrict__ phi, const double* __restrict__ ini,
                           double* __restrict__ L) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y, z = blockIdx.z;
    const int c[3] = {x, y, z};
    if (x >= g.n[0] || y >= g.n[1] || !is_interior(g, c)) return;
    const long long I = lin(g, x, y, z);
    const double s = sgn(ini[I]);
    double acc = 0.0;
    for (int i = 0; i < g.D; ++i) {
        const long long si = g.s[i];
        const int ci = c[i], n = g.n[i];
        double a, b = phi[I - si], cc = phi[I], d = phi[I + si], e;
        if (ci == 1) {                                   // lowerL!
            a = g.isper(i) ? phi[I + (long long)(n - 3 - ci) * si] : b;
            e = phi[I + 2 * si];
        } else if (ci == n - 2) {                        // upperL!
            a = phi[I - 2 * si];
            e = g.isper(i) ? phi[I + (long long)(2 - ci) * si] : d;
        } else {
            a = phi[I - 2 * si];
            e = phi[I + 2 * si];
        }
        acc += grad2(a, b, cc, d, e, s);
    }
    L[I] = ini[I] * (1.0 - sqrt(acc));
}

// ϕ = α ϕ⁰ + (1-α)(ϕ + dτ L) on interior cells
__global__ void stage_k(Grid g, double* __restrict__ phi, const double* __restrict__ phi0,
                        const double* __restrict__ L, double dtau, double alpha) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y, z = blockIdx.z;
    const int c[3] = {x, y, z};
    if (x >= g.n[0] || y >= g.n[1] || !is_interior(g, c)) return;
    const long long I = lin(g, x, y, z);
    phi[I] = alpha * phi0[I] + (1.0 - alpha) * (phi[I] + dtau * L[I]);
}

// ϕ = 2f - 1 and ϕini = ϕ on every cell (ghosts included, as the broadcast does)
__global__ void lsinit_k(long long n, const double* __restrict__ f, double* __restrict__ phi,
                         double* __restrict__ ini) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const double v = 2.0 * f[q] - 1.0;
        phi[q] = v;
        if (ini) ini[q] = v;
    }
}

}  // namespace
}  // namespace ia

using namespace ia;

extern "C" {

int ia_levelset_init(ia_handle* h, const double* f, double* phi, double* phi_ini) {
    if (!h || !f || !phi) return IA_ERR_INVALID;
    { lsinit_k<<<1216, 256, 0, h->stream>>>(h->g.N, f, phi, phi_ini); ia::note_launch(); }
    return cuda_fail(cudaGetLastError());
}

int ia_levelset_rhs(ia_handle* h, double* L, const double* phi, const double* phi_ini) {
    if (!h || !L || !phi || !phi_ini) return IA_ERR_INVALID;
    cudaMemsetAsync(L, 0, sizeof(double) * (size_t)h->g.N, h->stream);
    { computeL_k<<<grd(h->g), blk(), 0, h->stream>>>(h->g, phi, phi_ini, L); ia::note_launch(); }
    return cuda_fail(cudaGetLastError());
}

int ia_redistance(ia_handle* h, double* phi, double* phi0, const double* phi_ini, double* L, double d, double dtau) {
    if (!h || !phi || !phi0 || !phi_ini || !L || !(dtau > 0.0) || !(d >= 0.0)) return IA_ERR_INVALID;
    const Grid& g = h->g;
    cudaStream_t st = h->stream;
    const long long itmx = std::llrint(d / dtau);   // Julia round: nearest, ties to even
    const double alphas[3] = {0.0, 3.0 / 4.0, 1.0 / 3.0};
    cudaMemsetAsync(L, 0, sizeof(double) * (size_t)g.N, st);
    for (long long it = 0; it < itmx; ++it) {
        cudaMemcpyAsync(phi0, phi, sizeof(double) * (size_t)g.N, cudaMemcpyDeviceToDevice, st);
        for (int k = 0; k < 3; ++k) {
            { computeL_k<<<grd(g), blk(), 0, st>>>(g, phi, phi_ini, L); ia::note_launch(); }
            { stage_k<<<grd(g), blk(), 0, st>>>(g, phi, phi0, L, dtau, alphas[k]); ia::note_launch(); }
            if (fill_ghosts_scalar(g, phi, st) != cudaSuccess) return IA_ERR_CUDA;
        }
    }
    return cuda_fail(cudaGetLastError());
}

}  // extern "C"
