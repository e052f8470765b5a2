// Step diagnostics of src/metrics.jl as fused domain sums: Σ ρkeI (metrics.jl:13-15),
// Σ ρuI for each component (:56-58), Σ ρgh (:23), and Σ EnsI (:32-39) when a vorticity field
// is given.  One pass over the interior cells, FP64, per-block partial sums reduced in a fixed
// order (deterministic).  getρ(I, f, λρ) = λρ + (1-λρ) f[I] (src/VOFutil.jl:166, 174).
#include <cuda_runtime.h>

#include "capi_internal.cuh"

namespace ia {
namespace {

constexpr int MT = 256;
constexpr int MB = 600;   // NQ * MB + NQ partials fit the handle's 4096-double reduction buffer
constexpr int NQ = 6;   // ke, pe, ens, ρu_0, ρu_1, ρu_2

struct MetricArgs {
    Grid g;
    const double* u;
    const double* f;
    const double* w;     // vorticity (3D: edge vector field, component last; 2D: scalar) or null
    double lrho, one_m;
    double U[3], gv[3], wl[3];
};

__device__ __forceinline__ double sq(double v) { return v * v; }

__global__ void metrics_k(MetricArgs a, double* __restrict__ partial) {
    const Grid& g = a.g;
    double acc[NQ] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    const int nxi = g.n[0] - 2, nyi = g.n[1] - 2;
    const int rows = nyi * (g.D == 3 ? g.n[2] - 2 : 1);
    // rows b, b + G, ...: (y, z) advance incrementally
    const int dy = int(gridDim.x) % nyi, dz = int(gridDim.x) / nyi;
    int y = 1 + int(blockIdx.x) % nyi, z = (g.D == 3 ? 1 : 0) + int(blockIdx.x) / nyi;
    for (int rw = blockIdx.x; rw < rows; rw += gridDim.x, y += dy, z += dz + (y > nyi ? 1 : 0), y -= (y > nyi ? nyi : 0)) {
        for (int x = 1 + threadIdx.x; x <= nxi; x += blockDim.x) {
            const long long I = lin(g, x, y, z);
            const double rho = a.lrho + a.one_m * a.f[I];
            const int c[3] = {x, y, z};
            double ke = 0.0, pe = 0.0;
            for (int i = 0; i < g.D; ++i) {
                const double lo = a.u[I + i * g.N] - a.U[i], hi = a.u[I + g.s[i] + i * g.N] - a.U[i];
                ke += sq(lo) + sq(hi);
                acc[3 + i] += 0.5 * (a.u[I + i * g.N] + a.u[I + g.s[i] + i * g.N] - 2.0 * a.U[i]) * rho;
                pe += a.gv[i] * ((double(c[i]) - 0.5) - a.wl[i]);   // loc(0,I) = I - 1.5 (1-based)
            }
            acc[0] += 0.25 * ke * rho;
            acc[1] += -rho * pe;
            if (a.w) {
                double e = 0.0;
                if (g.D == 3) {
                    for (int i = 0; i < 3; ++i) {
                        const long long sx = g.s[(i + 1) % 3], sy = g.s[(i + 2) % 3];   // shiftDir(i,3,1/2)
                        const double* w = a.w + i * g.N;
                        e += sq(w[I]) + sq(w[I + sx]) + sq(w[I + sy]) + sq(w[I + sx + sy]);
                    }
                } else {
                    e = sq(a.w[I]) + sq(a.w[I + g.s[0]]) + sq(a.w[I + g.s[1]]) + sq(a.w[I + g.s[0] + g.s[1]]);
                }
                acc[2] += 0.5 * 0.25 * e;
            }
        }
    }
    __shared__ double sm[MT];
    for (int q = 0; q < NQ; ++q) {
        sm[threadIdx.x] = acc[q];
        __syncthreads();
        for (int w = MT / 2; w > 0; w >>= 1) {
            if (threadIdx.x < w) sm[threadIdx.x] += sm[threadIdx.x + w];
            __syncthreads();
        }
        if (threadIdx.x == 0) partial[q * gridDim.x + blockIdx.x] = sm[0];
        __syncthreads();
    }
}

__global__ void metrics_sum_k(const double* __restrict__ partial, int nb, double* __restrict__ out) {
    __shared__ double sm[MT];
    for (int q = 0; q < NQ; ++q) {
        double s = 0.0;
        for (int i = threadIdx.x; i < nb; i += blockDim.x) s += partial[q * nb + i];
        sm[threadIdx.x] = s;
        __syncthreads();
        for (int w = MT / 2; w > 0; w >>= 1) {
            if (threadIdx.x < w) sm[threadIdx.x] += sm[threadIdx.x + w];
            __syncthreads();
        }
        if (threadIdx.x == 0) out[q] = sm[0];
        __syncthreads();
    }
}

}  // namespace
}  // namespace ia

using namespace ia;

extern "C" int ia_metrics(ia_handle* h, const double* u, const double* f, const double* omega, const double* U,
                          const double* g, const double* statwl, double* out) {
    if (!h || !u || !f || !out) return IA_ERR_INVALID;
    MetricArgs a;
    a.g = h->g;
    a.u = u;
    a.f = f;
    a.w = omega;
    a.lrho = h->cfg.lrho;
    a.one_m = 1.0 - h->cfg.lrho;
    for (int i = 0; i < 3; ++i) {
        a.U[i] = (U && i < h->g.D) ? U[i] : 0.0;
        a.gv[i] = (g && i < h->g.D) ? g[i] : 0.0;
        a.wl[i] = (statwl && i < h->g.D) ? statwl[i] : 0.0;
    }
    const long long rows = (long long)(h->g.n[1] - 2) * (h->g.D == 3 ? h->g.n[2] - 2 : 1);
    const int nb = int(rows < MB ? rows : MB);
    double* part = h->partial;
    double* dout = part + (size_t)NQ * nb;
    { metrics_k<<<nb, MT, 0, h->stream>>>(a, part); ia::note_launch(); }
    { metrics_sum_k<<<1, MT, 0, h->stream>>>(part, nb, dout); ia::note_launch(); }
    double hout[NQ];
    cudaError_t e = cudaMemcpyAsync(hout, dout, sizeof(hout), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return IA_ERR_CUDA;
    out[0] = hout[0];
    out[1] = hout[1];
    out[2] = hout[2];
    for (int i = 0; i < h->g.D; ++i) out[3 + i] = hout[3 + i];
    return IA_OK;
}
