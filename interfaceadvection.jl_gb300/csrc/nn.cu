// Learned Poisson preconditioner (see nn.cuh for the network).
//
//  * Training kernels (FP32, CUDA cores): direct 3x3x3 convolution forward,
//    backward-data (flipped, transposed taps), backward-weight (per-tap block
//    reductions), pooling / upsampling / ReLU / skip adjoints, MSE loss, Adam.
//  * Inference kernel (BF16 weights and activations, FP32 accumulation on the
//    5th-generation tensor cores): implicit GEMM with M = 128 output cells,
//    N = Cout, K = 27 taps x Cin.  Per tap the 128 x Cin im2col tile is staged in
//    shared memory in the canonical K-major core-matrix layout; one elected
//    thread issues tcgen05.mma (kind::f16, BF16 x BF16 -> FP32 in TMEM) and
//    tcgen05.commit to a per-stage mbarrier; the four warps read the 128 x Cout
//    accumulator back with tcgen05.ld for the bias / ReLU / skip epilogue.
//    Every mbarrier wait is bounded; on timeout the kernel raises an error flag,
//    releases its TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "capi_internal.cuh"
#include "nn.cuh"

namespace ia {
namespace nn {

// ------------------------------------------------------------------ activation tensors
// storage [B][nz+2][ny+2][nx+2][C], interior cells (x, y, z) in 0..n-1
struct Dims {
    int B, nx, ny, nz;
    __host__ __device__ long long cells() const { return (long long)B * nx * ny * nz; }
    __host__ __device__ long long padded() const { return (long long)B * (nx + 2) * (ny + 2) * (nz + 2); }
    __host__ __device__ long long pos(int b, int x, int y, int z) const {
        return (((long long)b * (nz + 2) + z + 1) * (ny + 2) + y + 1) * (nx + 2) + x + 1;
    }
    __host__ __device__ void decode(long long q, int& b, int& x, int& y, int& z) const {
        x = int(q % nx);
        q /= nx;
        y = int(q % ny);
        q /= ny;
        z = int(q % nz);
        b = int(q / nz);
    }
    __host__ __device__ long long tap(int t) const {   // offset of tap t = (dz+1)*9 + (dy+1)*3 + (dx+1)
        const int dx = t % 3 - 1, dy = (t / 3) % 3 - 1, dz = t / 9 - 1;
        return ((long long)dz * (ny + 2) + dy) * (nx + 2) + dx;
    }
    __host__ __device__ Dims half() const { return Dims{B, nx / 2, ny / 2, nz / 2}; }
};

__device__ __forceinline__ long long child_pos(const Dims& f, int b, int X, int Y, int Z, int k) {
    return f.pos(b, 2 * X + (k & 1), 2 * Y + ((k >> 1) & 1), 2 * Z + (k >> 2));
}

#define FOR_CELLS(D)                                                                                      \
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < (D).cells();                \
         q += (long long)gridDim.x * blockDim.x)

// ------------------------------------------------------------------ FP32 training kernels
template <int CI, int CO>
__global__ void conv_fwd_f32(Dims d, const float* __restrict__ X, const float* __restrict__ W,
                             const float* __restrict__ bias, float* __restrict__ Z, float* __restrict__ A,
                             const float* __restrict__ skip, int relu) {
    FOR_CELLS(d) {
        int b, x, y, z;
        d.decode(q, b, x, y, z);
        const long long p = d.pos(b, x, y, z);
        float acc[CO];
#pragma unroll
        for (int o = 0; o < CO; ++o) acc[o] = __ldg(bias + o);
        for (int t = 0; t < 27; ++t) {
            const float* xp = X + (p + d.tap(t)) * CI;
            const float* wt = W + (long long)t * CO * CI;
#pragma unroll 4
            for (int c = 0; c < CI; ++c) {
                const float xv = xp[c];
#pragma unroll
                for (int o = 0; o < CO; ++o) acc[o] = fmaf(__ldg(wt + o * CI + c), xv, acc[o]);
            }
        }
#pragma unroll
        for (int o = 0; o < CO; ++o) {
            if (Z) Z[p * CO + o] = acc[o];
            float v = relu ? fmaxf(acc[o], 0.f) : acc[o];
            if (skip) v += skip[p * CO + o];
            A[p * CO + o] = v;
        }
    }
}

// dX[p] = Σ_t W[t]^T dY[p - off(t)]
template <int CI, int CO>
__global__ void conv_bwd_data_f32(Dims d, const float* __restrict__ dY, const float* __restrict__ W,
                                  float* __restrict__ dX) {
    FOR_CELLS(d) {
        int b, x, y, z;
        d.decode(q, b, x, y, z);
        const long long p = d.pos(b, x, y, z);
        float acc[CI];
#pragma unroll
        for (int c = 0; c < CI; ++c) acc[c] = 0.f;
        for (int t = 0; t < 27; ++t) {
            const float* yp = dY + (p - d.tap(t)) * CO;
            const float* wt = W + (long long)t * CO * CI;
#pragma unroll 4
            for (int o = 0; o < CO; ++o) {
                const float g = yp[o];
#pragma unroll
                for (int c = 0; c < CI; ++c) acc[c] = fmaf(__ldg(wt + o * CI + c), g, acc[c]);
            }
        }
#pragma unroll
        for (int c = 0; c < CI; ++c) dX[p * CI + c] = acc[c];
    }
}

// dW[t][o][c] += Σ_p X[p+off(t)][c] dY[p][o] over a chunk of cells (one tap per blockIdx.y);
// the tap-0 blocks also accumulate the bias gradient db[o] += Σ_p dY[p][o].
template <int CI, int CO>
__global__ void conv_bwd_w_f32(Dims d, const float* __restrict__ X, const float* __restrict__ dY,
                               float* __restrict__ dW, float* __restrict__ db, long long chunk) {
    constexpr int TILE = 32;
    constexpr int PAIRS = CI * CO;
    constexpr int PER = (PAIRS + 255) / 256;
    __shared__ float xs[TILE][CI];
    __shared__ float ys[TILE][CO];
    const int t = blockIdx.y;
    const long long toff = d.tap(t);
    const long long c0 = (long long)blockIdx.x * chunk;
    const long long c1 = min(d.cells(), c0 + chunk);
    float acc[PER];
#pragma unroll
    for (int k = 0; k < PER; ++k) acc[k] = 0.f;
    float bacc = 0.f;
    for (long long base = c0; base < c1; base += TILE) {
        for (int e = threadIdx.x; e < TILE * (CI + CO); e += blockDim.x) {
            const int r = e / (CI + CO), c = e % (CI + CO);
            const long long qq = base + r;
            float v = 0.f;
            if (qq < c1) {
                int b, x, y, z;
                d.decode(qq, b, x, y, z);
                const long long p = d.pos(b, x, y, z);
                v = (c < CI) ? X[(p + toff) * CI + c] : dY[p * CO + (c - CI)];
            }
            if (c < CI) xs[r][c] = v;
            else ys[r][c - CI] = v;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < PER; ++k) {
            const int pr = threadIdx.x + 256 * k;
            if (pr < PAIRS) {
                const int o = pr / CI, c = pr % CI;
                float sacc = acc[k];
                for (int r = 0; r < TILE; ++r) sacc = fmaf(xs[r][c], ys[r][o], sacc);
                acc[k] = sacc;
            }
        }
        if (t == 0 && threadIdx.x < CO)
            for (int r = 0; r < TILE; ++r) bacc += ys[r][threadIdx.x];
        __syncthreads();
    }
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        const int pr = threadIdx.x + 256 * k;
        if (pr < PAIRS) atomicAdd(dW + (long long)t * PAIRS + pr, acc[k]);
    }
    if (t == 0 && threadIdx.x < CO) atomicAdd(db + threadIdx.x, bacc);
}

// dZ = dA · [Z > 0]
__global__ void relu_bwd_f32(Dims d, int C, const float* __restrict__ Z, const float* __restrict__ dA,
                             float* __restrict__ dZ) {
    FOR_CELLS(d) {
        int b, x, y, z;
        d.decode(q, b, x, y, z);
        const long long p = d.pos(b, x, y, z) * C;
        for (int c = 0; c < C; ++c) dZ[p + c] = Z[p + c] > 0.f ? dA[p + c] : 0.f;
    }
}

// out (coarse dims dc) = mean of the 8 children of in (fine dims 2dc)
__global__ void pool_fwd_f32(Dims dc, int C, const float* __restrict__ in, float* __restrict__ out) {
    const Dims df{dc.B, 2 * dc.nx, 2 * dc.ny, 2 * dc.nz};
    FOR_CELLS(dc) {
        int b, x, y, z;
        dc.decode(q, b, x, y, z);
        const long long P = dc.pos(b, x, y, z) * C;
        for (int c = 0; c < C; ++c) {
            float s = 0.f;
            for (int k = 0; k < 8; ++k) s += in[child_pos(df, b, x, y, z, k) * C + c];
            out[P + c] = s * 0.125f;
        }
    }
}
// dIn[child] += dOut[parent] / 8   (fine dims df)
__global__ void pool_bwd_add_f32(Dims df, int C, const float* __restrict__ dout, float* __restrict__ din) {
    const Dims dc = df.half();
    FOR_CELLS(df) {
        int b, x, y, z;
        df.decode(q, b, x, y, z);
        const long long p = df.pos(b, x, y, z) * C, P = dc.pos(b, x / 2, y / 2, z / 2) * C;
        for (int c = 0; c < C; ++c) din[p + c] += 0.125f * dout[P + c];
    }
}
// out[child] = in[parent] (+ skip[child])  (fine dims df)
__global__ void up_fwd_f32(Dims df, int C, const float* __restrict__ in, const float* __restrict__ skip,
                           float* __restrict__ out) {
    const Dims dc = df.half();
    FOR_CELLS(df) {
        int b, x, y, z;
        df.decode(q, b, x, y, z);
        const long long p = df.pos(b, x, y, z) * C, P = dc.pos(b, x / 2, y / 2, z / 2) * C;
        for (int c = 0; c < C; ++c) out[p + c] = in[P + c] + (skip ? skip[p + c] : 0.f);
    }
}
// dIn[parent] = Σ children dOut  (coarse dims dc)
__global__ void up_bwd_f32(Dims dc, int C, const float* __restrict__ dout, float* __restrict__ din) {
    const Dims df{dc.B, 2 * dc.nx, 2 * dc.ny, 2 * dc.nz};
    FOR_CELLS(dc) {
        int b, x, y, z;
        dc.decode(q, b, x, y, z);
        const long long P = dc.pos(b, x, y, z) * C;
        for (int c = 0; c < C; ++c) {
            float s = 0.f;
            for (int k = 0; k < 8; ++k) s += dout[child_pos(df, b, x, y, z, k) * C + c];
            din[P + c] = s;
        }
    }
}

// dOut = 2 (out - tgt) / n ; loss partials
__global__ void mse_k(Dims d, const float* __restrict__ out, const float* __restrict__ tgt, float* __restrict__ dout,
                      double* __restrict__ loss) {
    __shared__ double sm[256];
    const double inv = 1.0 / double(d.cells());
    double s = 0.0;
    FOR_CELLS(d) {
        int b, x, y, z;
        d.decode(q, b, x, y, z);
        const long long p = d.pos(b, x, y, z);
        const float e = out[p] - tgt[p];
        dout[p] = float(2.0 * inv) * e;
        s += double(e) * double(e);
    }
    sm[threadIdx.x] = s;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) sm[threadIdx.x] += sm[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(loss, sm[0] * inv);
}

// Energy norm of the error with the patch's own coefficients: δ = out - tgt,
// E = Σ_p Σ_d c[p,d] (δ[p] - δ[p-e_d])² / n with c = input channel 1+d (λρ·L on the cell's lower
// d-face; zero on walls and in the halo, where δ is zero too); dout = dE/dout.
__global__ void energy_k(Dims d, const float* __restrict__ out, const float* __restrict__ tgt,
                         const float* __restrict__ x0, float* __restrict__ dout, double* __restrict__ loss) {
    __shared__ double sm[256];
    const double inv = 1.0 / double(d.cells());
    const long long off[3] = {1, (long long)(d.nx + 2), (long long)(d.nx + 2) * (d.ny + 2)};
    double acc = 0.0;
    FOR_CELLS(d) {
        int b, x, y, z;
        d.decode(q, b, x, y, z);
        const long long p = d.pos(b, x, y, z);
        const float dp = out[p] - tgt[p];
        float g = 0.f;
        for (int k = 0; k < 3; ++k) {
            const long long lo = p - off[k], hi = p + off[k];
            const float dl = dp - (out[lo] - tgt[lo]);          // across the lower face
            const float dh = (out[hi] - tgt[hi]) - dp;          // across the upper face
            const float cl = x0[p * 4 + 1 + k], ch = x0[hi * 4 + 1 + k];
            acc += double(cl) * double(dl) * double(dl);
            g += cl * dl - ch * dh;
        }
        dout[p] = float(2.0 * inv) * g;
    }
    sm[threadIdx.x] = acc;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) sm[threadIdx.x] += sm[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(loss, sm[0] * inv);
}

__global__ void adam_k(long long n, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

__global__ void zero_f32(long long n, float* a) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        a[i] = 0.f;
}

// ------------------------------------------------------------------ tcgen05 inference convolution
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor, K-major, no swizzle: core matrices of 8 rows x 16 bytes,
// LBO = byte distance of K-adjacent core matrices, SBO = of M/N-adjacent ones
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;   // descriptor version of the 5th-generation tensor cores
    return d;                 // base offset 0, layout SWIZZLE_NONE
}
// instruction descriptor, kind::f16: D F32, A/B BF16, both K-major
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Poll an mbarrier phase for at most ~1 s of wall time (and a fixed number of polls).
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
    const uint64_t t0 = global_ns();
    for (uint32_t i = 0; i < (1u << 28); ++i) {
        uint32_t ok = 0;
        asm volatile(
            "{\n\t.reg .pred P;\n\tmbarrier.try_wait.parity.shared::cta.b64 P, [%1], %2;\n\tselp.b32 %0, 1, 0, P;\n\t}\n"
            : "=r"(ok)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (ok) return true;
        if ((i & 255u) == 255u && global_ns() - t0 > 1000000000ull) return false;
    }
    return false;
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// ------------------------------------------------------------------ TMA-fed tensor-core convolution
// Inference activations are stored as 8-channel planes: plane j holds channels 8j..8j+7 of every
// (padded, halo-included) cell, 16 B per cell, so a run of cells of one plane is contiguous.
// A tile is M = 128 consecutive cells of one x-row (rows shorter than 128 leave the tail masked).
// For each of the 9 (dy, dz) neighbour rows and each plane, one TMA box of WR = 136 consecutive
// cells (2176 contiguous bytes) lands in shared memory as 136 rows of 16 B: the chunk column of a
// K-major no-swizzle operand whose 8-row core matrices are contiguous (SBO 128 B) and whose
// K-neighbour chunks are one box apart (LBO = 2176 B).  The A operand of tap (dx, dy, dz) is the
// (dy, dz) window started dx + 1 rows in, so all 27 taps are read from one set of 9·Cin/8 boxes.
// Two stages: thread 0 issues the next tile's boxes before the MMAs of this one; one commit per
// tile releases the epilogue (all four warps, tcgen05.ld) and the stage.
constexpr int kM = 128;   // output cells per tile (the MMA M)
constexpr int WR = 136;
constexpr int BOX_BYTES = WR * 16;

template <int CI, int COP>
struct TmaSmem {
    static constexpr int W_BYTES = 27 * COP * CI * 2;
    static constexpr int NBOX = 9 * (CI / 8);
    static constexpr int STAGE_BYTES = NBOX * BOX_BYTES;
    static constexpr int A_OFF = (W_BYTES + 1023) / 1024 * 1024;
    static constexpr int BAR_OFF = A_OFF + 2 * STAGE_BYTES;
    static constexpr int TOTAL = BAR_OFF + 64;
};

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int c0, int c1, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(bar)
        : "memory");
}

template <int CI, int CO, bool RELU, bool OUTF32>
__global__ void __launch_bounds__(128) conv_tma_kernel(const __grid_constant__ CUtensorMap tmap, Dims d,
                                                       const uint8_t* __restrict__ Wg, const float* __restrict__ bias,
                                                       const __nv_bfloat16* __restrict__ skip,
                                                       __nv_bfloat16* __restrict__ Y, float* __restrict__ Yf,
                                                       int* __restrict__ err) {
    constexpr int COP = CO < 16 ? 16 : CO;
    using S = TmaSmem<CI, COP>;
    static_assert(CI % 16 == 0 && COP % 16 == 0 && COP <= 32, "tile shape");
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint32_t tmem_holder;
    const int tid = threadIdx.x, warp = tid >> 5;
    for (int i = tid; i < S::W_BYTES / 16; i += blockDim.x)
        reinterpret_cast<uint4*>(smem)[i] = __ldg(reinterpret_cast<const uint4*>(Wg) + i);
    const uint32_t full0 = smem_u32(smem + S::BAR_OFF), mdone = full0 + 16;
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(full0));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(full0 + 8));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mdone));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_holder)),
                     "r"(32));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // weights: generic writes, async reads
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_holder;
    const uint32_t wbase = smem_u32(smem), abase = smem_u32(smem + S::A_OFF);
    constexpr uint32_t idesc = idesc_bf16(kM, COP);
    const int xtiles = (d.nx + kM - 1) / kM;
    const long long ntiles = (long long)xtiles * d.ny * d.nz * d.B;
    const int rowp = d.nx + 2;
    const long long planep = (long long)(d.nx + 2) * (d.ny + 2);
    const long long plane = d.padded() * 8;   // elements per 8-channel plane
    float bias_r[CO];
#pragma unroll
    for (int o = 0; o < CO; ++o) bias_r[o] = __ldg(bias + o);

    auto tile_origin = [&](long long t, int& x0) -> long long {
        x0 = int(t % xtiles) * kM;
        long long r = t / xtiles;
        const int y = int(r % d.ny);
        r /= d.ny;
        const int z = int(r % d.nz);
        const int b = int(r / d.nz);
        return d.pos(b, x0, y, z);
    };
    auto issue = [&](long long t, int s) {   // thread 0
        int x0;
        const long long p0 = tile_origin(t, x0);
        const uint32_t bar = full0 + 8 * s;
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(S::STAGE_BYTES)
                     : "memory");
        for (int w = 0; w < 9; ++w) {
            const long long row = p0 - 1 + (long long)(w % 3 - 1) * rowp + (long long)(w / 3 - 1) * planep;
#pragma unroll
            for (int j = 0; j < CI / 8; ++j)
                tma_load_2d(abase + s * S::STAGE_BYTES + (w * (CI / 8) + j) * BOX_BYTES, &tmap, 0,
                            int(row + (long long)j * d.padded()), bar);
        }
    };
    int issued[2] = {0, 0}, waited[2] = {0, 0}, commits = 0, commits_waited = 0;
    if (tid == 0 && (long long)blockIdx.x < ntiles) issue(blockIdx.x, 0);
    if ((long long)blockIdx.x < ntiles) issued[0] = 1;
    bool failed = false;
    int i = 0;
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++i) {
        const int s = i & 1;
        const long long next = tile + gridDim.x;
        if (next < ntiles) {
            if (tid == 0) issue(next, s ^ 1);
            issued[s ^ 1] += 1;
        }
        bool ok = mbar_wait(full0 + 8 * s, uint32_t((i >> 1) & 1));
        if (__syncthreads_or(!ok)) {
            failed = true;
            break;
        }
        waited[s] += 1;
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t st = abase + s * S::STAGE_BYTES;
#pragma unroll 1
            for (int t = 0; t < 27; ++t) {
                const int w = t / 3, dx1 = t % 3;   // window (dy, dz) and dx + 1
#pragma unroll
                for (int ks = 0; ks < CI / 16; ++ks) {
                    const uint64_t ad =
                        smem_desc(st + (w * (CI / 8) + 2 * ks) * BOX_BYTES + dx1 * 16, BOX_BYTES, 128);
                    const uint64_t bd = smem_desc(wbase + t * COP * CI * 2 + ks * 256, 128, CI * 16);
                    const uint32_t acc = (t > 0 || ks > 0) ? 1u : 0u;
                    asm volatile(
                        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
                        "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
                }
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mdone)
                         : "memory");
        }
        ++commits;
        ok = mbar_wait(mdone, uint32_t(i & 1));
        if (__syncthreads_or(!ok)) {
            failed = true;
            break;
        }
        ++commits_waited;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        int x0;
        const long long p0 = tile_origin(tile, x0);
        const bool valid = x0 + tid < d.nx;
        const long long p = p0 + tid;
        const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
        if (OUTF32) {
            float v[16];
            tmem_ld16(trow, v);
            if (valid) Yf[p] = v[0] + bias_r[0];
        } else {
#pragma unroll
            for (int c0 = 0; c0 < CO; c0 += 16) {
                float v[16];
                tmem_ld16(trow + c0, v);
                if (valid) {
                    uint32_t packed[8];
#pragma unroll
                    for (int k = 0; k < 16; k += 2) {
                        float a = v[k] + bias_r[c0 + k], b2 = v[k + 1] + bias_r[c0 + k + 1];
                        if (RELU) {
                            a = fmaxf(a, 0.f);
                            b2 = fmaxf(b2, 0.f);
                        }
                        if (skip) {
                            const long long sp = (long long)((c0 + k) / 8) * plane + p * 8 + (k % 8);
                            const __nv_bfloat162 sk = *reinterpret_cast<const __nv_bfloat162*>(skip + sp);
                            a += __low2float(sk);
                            b2 += __high2float(sk);
                        }
                        const __nv_bfloat162 o2 = __floats2bfloat162_rn(a, b2);
                        packed[k / 2] = *reinterpret_cast<const uint32_t*>(&o2);
                    }
                    *reinterpret_cast<uint4*>(Y + (long long)(c0 / 8) * plane + p * 8) =
                        make_uint4(packed[0], packed[1], packed[2], packed[3]);
                    *reinterpret_cast<uint4*>(Y + (long long)(c0 / 8 + 1) * plane + p * 8) =
                        make_uint4(packed[4], packed[5], packed[6], packed[7]);
                }
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
    }
    if (failed) {
        if (tid == 0) atomicExch(err, 1);
        // bounded drain: the last commit and every box load still in flight
        if (commits > commits_waited) mbar_wait(mdone, uint32_t((commits - 1) & 1));
        for (int s = 0; s < 2; ++s)
            if (issued[s] > waited[s]) mbar_wait(full0 + 8 * s, uint32_t((issued[s] - 1) & 1));
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(32));
}

// ------------------------------------------------------------------ BF16 glue kernels (inference)
// 8-channel planes: element (cell p, channel c) at (c/8)·8·padded + 8p + c%8; 16 B per cell and plane
__device__ __forceinline__ void acc8(float (&a)[8], const uint4& v) {
    const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&v);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        a[2 * i] += __low2float(h[i]);
        a[2 * i + 1] += __high2float(h[i]);
    }
}
__device__ __forceinline__ uint4 pack8(const float (&a)[8]) {
    uint4 v;
    __nv_bfloat162* h = reinterpret_cast<__nv_bfloat162*>(&v);
#pragma unroll
    for (int i = 0; i < 4; ++i) h[i] = __floats2bfloat162_rn(a[2 * i], a[2 * i + 1]);
    return v;
}

// out (coarse dims dc) = mean of the 8 children of in (fine dims 2dc), C/8 planes
__global__ void pool_bf16(Dims dc, int C, const __nv_bfloat16* __restrict__ in, __nv_bfloat16* __restrict__ out) {
    const Dims df{dc.B, 2 * dc.nx, 2 * dc.ny, 2 * dc.nz};
    const long long pin = df.padded() * 8, pout = dc.padded() * 8;
    FOR_CELLS(dc) {
        int b, x, y, z;
        dc.decode(q, b, x, y, z);
        const long long P = dc.pos(b, x, y, z);
        for (int j = 0; j < C / 8; ++j) {
            float a[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            for (int k = 0; k < 8; ++k)
                acc8(a, *reinterpret_cast<const uint4*>(in + j * pin + child_pos(df, b, x, y, z, k) * 8));
#pragma unroll
            for (int i = 0; i < 8; ++i) a[i] *= 0.125f;
            *reinterpret_cast<uint4*>(out + j * pout + P * 8) = pack8(a);
        }
    }
}
// out[child] = in[parent] (+ skip[child])  (fine dims df), C/8 planes
__global__ void up_bf16(Dims df, int C, const __nv_bfloat16* __restrict__ in, const __nv_bfloat16* __restrict__ skip,
                        __nv_bfloat16* __restrict__ out) {
    const Dims dc = df.half();
    const long long pf = df.padded() * 8, pc = dc.padded() * 8;
    FOR_CELLS(df) {
        int b, x, y, z;
        df.decode(q, b, x, y, z);
        const long long p = df.pos(b, x, y, z), P = dc.pos(b, x / 2, y / 2, z / 2);
        for (int j = 0; j < C / 8; ++j) {
            const uint4 v = *reinterpret_cast<const uint4*>(in + j * pc + P * 8);
            if (skip) {
                float a[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
                acc8(a, v);
                acc8(a, *reinterpret_cast<const uint4*>(skip + j * pf + p * 8));
                *reinterpret_cast<uint4*>(out + j * pf + p * 8) = pack8(a);
            } else {
                *reinterpret_cast<uint4*>(out + j * pf + p * 8) = v;
            }
        }
    }
}
// FP32 4-channel input (training layout) -> BF16 planes 0 (channels 0-3, 4-7 zero) and 1 (zero)
__global__ void in_to_bf16(Dims d, const float* __restrict__ x4, __nv_bfloat16* __restrict__ x16) {
    const long long pl = d.padded() * 8;
    FOR_CELLS(d) {
        int b, x, y, z;
        d.decode(q, b, x, y, z);
        const long long p = d.pos(b, x, y, z);
        const float4 v = *reinterpret_cast<const float4*>(x4 + p * 4);
        const float a[8] = {v.x, v.y, v.z, v.w, 0.f, 0.f, 0.f, 0.f};
        *reinterpret_cast<uint4*>(x16 + p * 8) = pack8(a);
        *reinterpret_cast<uint4*>(x16 + pl + p * 8) = make_uint4(0u, 0u, 0u, 0u);
    }
}

// ---- preconditioner input from the solver's grid arrays.  The padded activation layout of
// a batch of one equals the solver's ghost-width-1 column-major grid layout, so the solver's
// residual, coefficients and the net output share one index p.
__global__ void absmax_k(Dims d, const float* __restrict__ r, unsigned int* __restrict__ out) {
    __shared__ unsigned int sm[256];
    unsigned int m = 0u;
    FOR_CELLS(d) {
        int b, x, y, z;
        d.decode(q, b, x, y, z);
        const unsigned int v = __float_as_uint(r[d.pos(b, x, y, z)]) & 0x7FFFFFFFu;
        m = v > m ? v : m;
    }
    sm[threadIdx.x] = m;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) sm[threadIdx.x] = sm[threadIdx.x] > sm[threadIdx.x + w] ? sm[threadIdx.x] : sm[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicMax(out, sm[0]);
}

// channels: r / max|r|, λρ·L_x, λρ·L_y, λρ·L_z (lower-face coefficients of the cell), zeros;
// written as 8-channel planes
__global__ void prep_k(Dims d, const float* __restrict__ r, const float* __restrict__ L, long long ncomp, float lrho,
                       const unsigned int* __restrict__ scale, __nv_bfloat16* __restrict__ x16) {
    const float sc = __uint_as_float(*scale);
    const float inv = sc > 0.f ? 1.f / sc : 0.f;
    FOR_CELLS(d) {
        int b, x, y, z;
        d.decode(q, b, x, y, z);
        const long long p = d.pos(b, x, y, z);
        const __nv_bfloat162 c01 = __floats2bfloat162_rn(r[p] * inv, lrho * L[p]);
        const __nv_bfloat162 c23 = __floats2bfloat162_rn(lrho * L[p + ncomp], lrho * L[p + 2 * ncomp]);
        // plane 0; plane 1 (channels 8-15) stays zero from the allocation
        *reinterpret_cast<uint4*>(x16 + p * 8) =
            make_uint4(*reinterpret_cast<const uint32_t*>(&c01), *reinterpret_cast<const uint32_t*>(&c23), 0u, 0u);
    }
}

}  // namespace nn

// ------------------------------------------------------------------ state
struct NNState {
    float *w = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;   // FP32 parameters, gradient, Adam moments
    long long step = 0;
    int loss_kind = 0;                                               // 0 MSE, 1 energy norm
    uint8_t* wtc[nn::NLAYER] = {nullptr};                            // BF16 weights, shared-memory layout
    float* bias_tc = nullptr;                                        // padded biases (16 or 32 per layer)
    bool tc_dirty = true;
    // training activations (FP32); zeroed whenever the dims change so every halo is zero
    float* buf = nullptr;
    size_t buf_bytes = 0;
    nn::Dims buf_dims{0, 0, 0, 0};
    // inference activations (BF16), same rule
    __nv_bfloat16* ibuf = nullptr;
    size_t ibuf_bytes = 0;
    nn::Dims ibuf_dims{0, 0, 0, 0};
    // preconditioner input (BF16, 16 channels, grid-shaped) and its scale
    __nv_bfloat16* x16 = nullptr;
    size_t x16_bytes = 0;
    unsigned int* dscale = nullptr;
    double* dloss = nullptr;
    int* derr = nullptr;
};

inline bool same_dims(const nn::Dims& a, const nn::Dims& b) {
    return a.B == b.B && a.nx == b.nx && a.ny == b.ny && a.nz == b.nz;
}

namespace {

NNState* nn_state(ia_handle* h) {
    if (h->nn) return h->nn;
    NNState* s = new NNState();
    const size_t n = (size_t)nn::NPARAM;
    cudaError_t e = cudaSuccess;
    e = e ? e : cudaMalloc(&s->w, 4 * n);
    e = e ? e : cudaMalloc(&s->g, 4 * n);
    e = e ? e : cudaMalloc(&s->m, 4 * n);
    e = e ? e : cudaMalloc(&s->v, 4 * n);
    e = e ? e : cudaMalloc(&s->dloss, 8);
    e = e ? e : cudaMalloc(&s->derr, 4);
    e = e ? e : cudaMalloc(&s->dscale, 4);
    e = e ? e : cudaMalloc(&s->bias_tc, 4 * 32 * nn::NLAYER);
    for (int l = 0; l < nn::NLAYER && !e; ++l) {
        const int co = nn::COUT[l] < 16 ? 16 : nn::COUT[l], ci = nn::CIN[l] < 16 ? 16 : nn::CIN[l];
        e = cudaMalloc(&s->wtc[l], (size_t)27 * co * ci * 2);
    }
    if (e != cudaSuccess) return nullptr;
    cudaMemset(s->w, 0, 4 * n);
    cudaMemset(s->m, 0, 4 * n);
    cudaMemset(s->v, 0, 4 * n);
    cudaMemset(s->derr, 0, 4);
    h->nn = s;
    return s;
}

float* take(float*& cur, long long n) {
    float* p = cur;
    cur += (n + 63) / 64 * 64;
    return p;
}

// padded tensor sizes (floats) of the training graph for dims d (full resolution)
struct Graph {
    nn::Dims f, hf, qt;
    float *x0, *z1, *a1, *p1, *z2, *a2, *p2, *z3, *a3, *u2, *z4, *a4, *u1, *z5, *a5, *out, *tgt;
    float *dout, *da5, *dz5, *du1, *da4, *dz4, *du2, *da3, *dz3, *dp2, *da2, *dz2, *dp1, *da1, *dz1;
};

size_t graph_floats(const nn::Dims& f) {
    const nn::Dims hf = f.half(), qt = hf.half();
    const long long F = f.padded(), H = hf.padded(), Q = qt.padded();
    const long long per = F * (4 + 16 * 3 + 32 + 16 * 2 + 1 + 1) + H * (16 + 32 * 5) + Q * (32 * 3) +
                          F * (1 + 16 * 2 + 32 + 16 * 2) + H * (16 + 32 * 5) + Q * (32 * 3);
    return (size_t)per + 64 * 40;
}

Graph carve(float* base, const nn::Dims& f) {
    Graph G;
    G.f = f;
    G.hf = f.half();
    G.qt = G.hf.half();
    const long long F = f.padded(), H = G.hf.padded(), Q = G.qt.padded();
    float* c = base;
    G.x0 = take(c, F * 4);
    G.z1 = take(c, F * 16);
    G.a1 = take(c, F * 16);
    G.p1 = take(c, H * 16);
    G.z2 = take(c, H * 32);
    G.a2 = take(c, H * 32);
    G.p2 = take(c, Q * 32);
    G.z3 = take(c, Q * 32);
    G.a3 = take(c, Q * 32);
    G.u2 = take(c, H * 32);
    G.z4 = take(c, H * 32);
    G.a4 = take(c, H * 32);
    G.u1 = take(c, F * 32);
    G.z5 = take(c, F * 16);
    G.a5 = take(c, F * 16);
    G.out = take(c, F);
    G.tgt = take(c, F);
    G.dout = take(c, F);
    G.da5 = take(c, F * 16);
    G.dz5 = take(c, F * 16);
    G.du1 = take(c, F * 32);
    G.da4 = take(c, H * 32);
    G.dz4 = take(c, H * 32);
    G.du2 = take(c, H * 32);
    G.da3 = take(c, Q * 32);
    G.dz3 = take(c, Q * 32);
    G.dp2 = take(c, Q * 32);
    G.da2 = take(c, H * 32);
    G.dz2 = take(c, H * 32);
    G.dp1 = take(c, H * 16);
    G.da1 = take(c, F * 16);
    G.dz1 = take(c, F * 16);
    return G;
}

int ensure_graph(ia_handle* h, NNState* s, const nn::Dims& f, Graph& G) {
    const size_t need = graph_floats(f) * 4;
    if (need > s->buf_bytes) {
        cudaFree(s->buf);
        s->buf = nullptr;
        s->buf_bytes = 0;
        s->buf_dims = nn::Dims{0, 0, 0, 0};
        if (cudaMalloc(&s->buf, need) != cudaSuccess) return IA_ERR_CUDA;
        s->buf_bytes = need;
    }
    if (!same_dims(f, s->buf_dims)) {
        if (cudaMemsetAsync(s->buf, 0, s->buf_bytes, h->stream) != cudaSuccess) return IA_ERR_CUDA;
        s->buf_dims = f;
    }
    G = carve(s->buf, f);
    return IA_OK;
}

inline int nblk(long long n) {
    long long b = (n + 255) / 256;
    return int(b < 4096 ? (b < 1 ? 1 : b) : 4096);
}

template <int CI, int CO>
void fwd(const nn::Dims& d, const float* X, const float* W, const float* b, float* Z, float* A, const float* skip,
         int relu, cudaStream_t st) {
    { nn::conv_fwd_f32<CI, CO><<<nblk(d.cells()), 256, 0, st>>>(d, X, W, b, Z, A, skip, relu); ia::note_launch(); }
}
template <int CI, int CO>
void bwd(const nn::Dims& d, const float* X, const float* dY, const float* W, float* dW, float* db, float* dX,
         cudaStream_t st) {
    // about 96 chunks per tap (27 x 96 blocks), at least 1024 cells each
    long long chunk = (d.cells() + 95) / 96;
    chunk = chunk < 1024 ? 1024 : (chunk + 31) / 32 * 32;
    const dim3 grid((unsigned)((d.cells() + chunk - 1) / chunk), 27);
    { nn::conv_bwd_w_f32<CI, CO><<<grid, 256, 0, st>>>(d, X, dY, dW, db, chunk); ia::note_launch(); }
    if (dX) { nn::conv_bwd_data_f32<CI, CO><<<nblk(d.cells()), 256, 0, st>>>(d, dY, W, dX); ia::note_launch(); }
}

// forward of the training graph (inputs already in G.x0)
void forward_f32(const Graph& G, const float* w, cudaStream_t st) {
    using namespace nn;
    fwd<4, 16>(G.f, G.x0, w + layer_w(0), w + layer_b(0), G.z1, G.a1, nullptr, 1, st);
    { pool_fwd_f32<<<nblk(G.hf.cells()), 256, 0, st>>>(G.hf, 16, G.a1, G.p1); ia::note_launch(); }
    fwd<16, 32>(G.hf, G.p1, w + layer_w(1), w + layer_b(1), G.z2, G.a2, nullptr, 1, st);
    { pool_fwd_f32<<<nblk(G.qt.cells()), 256, 0, st>>>(G.qt, 32, G.a2, G.p2); ia::note_launch(); }
    fwd<32, 32>(G.qt, G.p2, w + layer_w(2), w + layer_b(2), G.z3, G.a3, nullptr, 1, st);
    { up_fwd_f32<<<nblk(G.hf.cells()), 256, 0, st>>>(G.hf, 32, G.a3, G.a2, G.u2); ia::note_launch(); }
    fwd<32, 32>(G.hf, G.u2, w + layer_w(3), w + layer_b(3), G.z4, G.a4, nullptr, 1, st);
    { up_fwd_f32<<<nblk(G.f.cells()), 256, 0, st>>>(G.f, 32, G.a4, nullptr, G.u1); ia::note_launch(); }
    fwd<32, 16>(G.f, G.u1, w + layer_w(4), w + layer_b(4), G.z5, G.a5, G.a1, 1, st);
    fwd<16, 1>(G.f, G.a5, w + layer_w(5), w + layer_b(5), nullptr, G.out, nullptr, 0, st);
}

void backward_f32(const Graph& G, const float* w, float* g, cudaStream_t st) {
    using namespace nn;
    bwd<16, 1>(G.f, G.a5, G.dout, w + layer_w(5), g + layer_w(5), g + layer_b(5), G.da5, st);
    { relu_bwd_f32<<<nblk(G.f.cells()), 256, 0, st>>>(G.f, 16, G.z5, G.da5, G.dz5); ia::note_launch(); }
    bwd<32, 16>(G.f, G.u1, G.dz5, w + layer_w(4), g + layer_w(4), g + layer_b(4), G.du1, st);
    { up_bwd_f32<<<nblk(G.hf.cells()), 256, 0, st>>>(G.hf, 32, G.du1, G.da4); ia::note_launch(); }
    { relu_bwd_f32<<<nblk(G.hf.cells()), 256, 0, st>>>(G.hf, 32, G.z4, G.da4, G.dz4); ia::note_launch(); }
    bwd<32, 32>(G.hf, G.u2, G.dz4, w + layer_w(3), g + layer_w(3), g + layer_b(3), G.du2, st);
    { up_bwd_f32<<<nblk(G.qt.cells()), 256, 0, st>>>(G.qt, 32, G.du2, G.da3); ia::note_launch(); }
    { relu_bwd_f32<<<nblk(G.qt.cells()), 256, 0, st>>>(G.qt, 32, G.z3, G.da3, G.dz3); ia::note_launch(); }
    bwd<32, 32>(G.qt, G.p2, G.dz3, w + layer_w(2), g + layer_w(2), g + layer_b(2), G.dp2, st);
    // da2 = du2 (skip) + pool adjoint of dp2
    cudaMemcpyAsync(G.da2, G.du2, sizeof(float) * G.hf.padded() * 32, cudaMemcpyDeviceToDevice, st);
    { pool_bwd_add_f32<<<nblk(G.hf.cells()), 256, 0, st>>>(G.hf, 32, G.dp2, G.da2); ia::note_launch(); }
    { relu_bwd_f32<<<nblk(G.hf.cells()), 256, 0, st>>>(G.hf, 32, G.z2, G.da2, G.dz2); ia::note_launch(); }
    bwd<16, 32>(G.hf, G.p1, G.dz2, w + layer_w(1), g + layer_w(1), g + layer_b(1), G.dp1, st);
    // da1 = da5 (skip) + pool adjoint of dp1
    cudaMemcpyAsync(G.da1, G.da5, sizeof(float) * G.f.padded() * 16, cudaMemcpyDeviceToDevice, st);
    { pool_bwd_add_f32<<<nblk(G.f.cells()), 256, 0, st>>>(G.f, 16, G.dp1, G.da1); ia::note_launch(); }
    { relu_bwd_f32<<<nblk(G.f.cells()), 256, 0, st>>>(G.f, 16, G.z1, G.da1, G.dz1); ia::note_launch(); }
    bwd<4, 16>(G.f, G.x0, G.dz1, w + layer_w(0), g + layer_w(0), g + layer_b(0), nullptr, st);
}

int loss_grad(ia_handle* h, NNState* s, const float* x0, const float* tgt, const nn::Dims& f, double* loss_out) {
    cudaStream_t st = h->stream;
    Graph G;
    if (ensure_graph(h, s, f, G) != IA_OK) return IA_ERR_CUDA;
    cudaMemcpyAsync(G.x0, x0, sizeof(float) * f.padded() * 4, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(G.tgt, tgt, sizeof(float) * f.padded(), cudaMemcpyDeviceToDevice, st);
    forward_f32(G, s->w, st);
    cudaMemsetAsync(s->dloss, 0, 8, st);
    const int nbl = nblk(f.cells()) < 1024 ? nblk(f.cells()) : 1024;
    if (s->loss_kind == 1) { nn::energy_k<<<nbl, 256, 0, st>>>(f, G.out, G.tgt, G.x0, G.dout, s->dloss); ia::note_launch(); }
    else { nn::mse_k<<<nbl, 256, 0, st>>>(f, G.out, G.tgt, G.dout, s->dloss); ia::note_launch(); }
    { nn::zero_f32<<<256, 256, 0, st>>>(nn::NPARAM, s->g); ia::note_launch(); }
    backward_f32(G, s->w, s->g, st);
    if (loss_out) {
        cudaMemcpyAsync(loss_out, s->dloss, 8, cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) return IA_ERR_CUDA;
    }
    return cudaGetLastError() == cudaSuccess ? IA_OK : IA_ERR_CUDA;
}

// FP32 parameters -> BF16 tiles in the tcgen05 shared-memory layout (host-side re-arrangement)
int build_tc_weights(ia_handle* h, NNState* s) {
    std::vector<float> w((size_t)nn::NPARAM);
    if (cudaMemcpy(w.data(), s->w, 4 * w.size(), cudaMemcpyDeviceToHost) != cudaSuccess) return IA_ERR_CUDA;
    std::vector<float> biases(32 * nn::NLAYER, 0.f);
    for (int l = 0; l < nn::NLAYER; ++l) {
        const int CI = nn::CIN[l], CO = nn::COUT[l];
        const int ci = CI < 16 ? 16 : CI, co = CO < 16 ? 16 : CO;
        const uint32_t SBO = ci * 16;
        std::vector<__nv_bfloat16> t((size_t)27 * co * ci, __float2bfloat16(0.f));
        for (int tap = 0; tap < 27; ++tap)
            for (int n = 0; n < CO; ++n)
                for (int k = 0; k < CI; ++k) {
                    const float v = w[nn::layer_w(l) + ((long long)tap * CO + n) * CI + k];
                    const size_t byte = (size_t)tap * co * ci * 2 + (n / 8) * SBO + (k / 8) * 128 + (n % 8) * 16 + (k % 8) * 2;
                    t[byte / 2] = __float2bfloat16(v);
                }
        if (cudaMemcpy(s->wtc[l], t.data(), t.size() * 2, cudaMemcpyHostToDevice) != cudaSuccess) return IA_ERR_CUDA;
        for (int n = 0; n < CO; ++n) biases[32 * l + n] = w[nn::layer_b(l) + n];
    }
    if (cudaMemcpy(s->bias_tc, biases.data(), 4 * biases.size(), cudaMemcpyHostToDevice) != cudaSuccess)
        return IA_ERR_CUDA;
    s->tc_dirty = false;
    return IA_OK;
}

// cuTensorMapEncodeTiled from the driver, without linking libcuda
using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiled encode_tiled() {
    static EncodeTiled fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess && q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiled>(p);
    }
    return fn;
}

// tensor map of a BF16 activation stored as Cin/8 planes of 8 channels: a 2D view of
// (Cin/8)·rows cells x 8 channels, box = 8 channels x WR cells; loads past either end read zeros
bool make_act_map(CUtensorMap* m, const __nv_bfloat16* X, int CI, long long rows) {
    EncodeTiled enc = encode_tiled();
    if (!enc) return false;
    const cuuint64_t dims[2] = {8, (cuuint64_t)rows * (CI / 8)};
    const cuuint64_t strides[1] = {16};
    const cuuint32_t box[2] = {8, (cuuint32_t)nn::WR};
    const cuuint32_t estr[2] = {1, 1};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<__nv_bfloat16*>(X), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int CI, int CO, bool RELU, bool OUTF32>
cudaError_t launch_tma(const nn::Dims& d, const __nv_bfloat16* X, const uint8_t* W, const float* b,
                       const __nv_bfloat16* skip, __nv_bfloat16* Y, float* Yf, int* err, cudaStream_t st, int sms) {
    using Sm = nn::TmaSmem<CI, CO < 16 ? 16 : CO>;
    CUtensorMap map;
    if (!make_act_map(&map, X, CI, d.padded())) return cudaErrorNotSupported;
    auto kfn = nn::conv_tma_kernel<CI, CO, RELU, OUTF32>;
    cudaError_t e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, Sm::TOTAL);
    if (e != cudaSuccess) return e;
    const long long tiles = (long long)((d.nx + nn::kM - 1) / nn::kM) * d.ny * d.nz * d.B;
    const int per_sm = Sm::TOTAL <= 110 * 1024 ? 2 : 1;
    const int grid = int(tiles < (long long)per_sm * sms ? tiles : (long long)per_sm * sms);
    { kfn<<<grid, 128, Sm::TOTAL, st>>>(map, d, W, b, skip, Y, Yf, err); ia::note_launch(); }
    return cudaGetLastError();
}

// one convolution layer of the inference path
#define conv_layer(CI_, CO_, RELU_, F32_, dims, X_, W_, B_, SK_, Y_, YF_) \
    launch_tma<CI_, CO_, RELU_, F32_>(dims, X_, W_, B_, SK_, Y_, YF_, s->derr, st, sms)

// inference with the tensor-core kernels; x16 = BF16 16-channel input, out = FP32 channel
int forward_tc(ia_handle* h, NNState* s, const nn::Dims& f, const __nv_bfloat16* x16, float* out) {
    cudaStream_t st = h->stream;
    if (s->tc_dirty && build_tc_weights(h, s) != IA_OK) return IA_ERR_CUDA;
    const nn::Dims hf = f.half(), qt = hf.half();
    const long long F = f.padded(), H = hf.padded(), Q = qt.padded();
    const size_t need = 2 * (size_t)(F * (16 + 32 + 16) + H * (16 + 32 * 3) + Q * (32 * 2) + 64 * 16);
    if (need > s->ibuf_bytes) {
        cudaFree(s->ibuf);
        s->ibuf = nullptr;
        s->ibuf_bytes = 0;
        s->ibuf_dims = nn::Dims{0, 0, 0, 0};
        if (cudaMalloc(&s->ibuf, need) != cudaSuccess) return IA_ERR_CUDA;
        s->ibuf_bytes = need;
    }
    if (!same_dims(f, s->ibuf_dims)) {   // halos must be zero: the kernels write interior cells only
        if (cudaMemsetAsync(s->ibuf, 0, s->ibuf_bytes, st) != cudaSuccess) return IA_ERR_CUDA;
        s->ibuf_dims = f;
    }
    __nv_bfloat16* c = s->ibuf;
    auto tk = [&](long long n) { __nv_bfloat16* p = c; c += (n + 63) / 64 * 64; return p; };
    __nv_bfloat16 *a1 = tk(F * 16), *u1 = tk(F * 32), *a5 = tk(F * 16), *p1 = tk(H * 16), *a2 = tk(H * 32),
                  *u2 = tk(H * 32), *a4 = tk(H * 32), *p2 = tk(Q * 32), *a3 = tk(Q * 32);
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device);
    const float* b = s->bias_tc;
    cudaError_t e = cudaSuccess;
    e = e ? e : conv_layer(16, 16, true, false, f, x16, s->wtc[0], b + 0, nullptr, a1, nullptr);
    if (!e) { nn::pool_bf16<<<nblk(hf.cells()), 256, 0, st>>>(hf, 16, a1, p1); ia::note_launch(); }
    e = e ? e : conv_layer(16, 32, true, false, hf, p1, s->wtc[1], b + 32, nullptr, a2, nullptr);
    if (!e) { nn::pool_bf16<<<nblk(qt.cells()), 256, 0, st>>>(qt, 32, a2, p2); ia::note_launch(); }
    e = e ? e : conv_layer(32, 32, true, false, qt, p2, s->wtc[2], b + 64, nullptr, a3, nullptr);
    if (!e) { nn::up_bf16<<<nblk(hf.cells()), 256, 0, st>>>(hf, 32, a3, a2, u2); ia::note_launch(); }
    e = e ? e : conv_layer(32, 32, true, false, hf, u2, s->wtc[3], b + 96, nullptr, a4, nullptr);
    if (!e) { nn::up_bf16<<<nblk(f.cells()), 256, 0, st>>>(f, 32, a4, nullptr, u1); ia::note_launch(); }
    e = e ? e : conv_layer(32, 16, true, false, f, u1, s->wtc[4], b + 128, a1, a5, nullptr);
    e = e ? e : conv_layer(16, 1, false, true, f, a5, s->wtc[5], b + 160, nullptr, nullptr, out);
    return e == cudaSuccess ? IA_OK : IA_ERR_CUDA;
}

int check_dims(int B, int nx, int ny, int nz) {
    if (B < 1 || nx < 4 || ny < 4 || nz < 4 || nx % 4 || ny % 4 || nz % 4) return IA_ERR_INVALID;
    return IA_OK;
}

}  // namespace

// Preconditioner application for the Poisson solver: out (FP32, grid layout, interior cells
// written) = net(r / max|r|, λρ·L) on a 3D grid with interior dims nx, ny, nz.
int nn_apply(ia_handle* h, const float* r, const float* L32, float* out, int nx, int ny, int nz, long long ncomp) {
    NNState* s = nn_state(h);
    if (!s) return IA_ERR_CUDA;
    cudaStream_t st = h->stream;
    const nn::Dims f{1, nx, ny, nz};
    const size_t need = 2 * 16 * (size_t)f.padded();
    if (need > s->x16_bytes) {
        cudaFree(s->x16);
        s->x16 = nullptr;
        s->x16_bytes = 0;
        if (cudaMalloc(&s->x16, need) != cudaSuccess) return IA_ERR_CUDA;
        s->x16_bytes = need;
        if (cudaMemsetAsync(s->x16, 0, need, st) != cudaSuccess) return IA_ERR_CUDA;
    }
    cudaMemsetAsync(s->dscale, 0, 4, st);
    const int nb = nblk(f.cells()) < 1216 ? nblk(f.cells()) : 1216;
    { nn::absmax_k<<<nb, 256, 0, st>>>(f, r, s->dscale); ia::note_launch(); }
    { nn::prep_k<<<nblk(f.cells()), 256, 0, st>>>(f, r, L32, ncomp, float(h->cfg.lrho), s->dscale, s->x16); ia::note_launch(); }
    return forward_tc(h, s, f, s->x16, out);
}
int nn_error_flag(ia_handle* h) {
    if (!h->nn) return 0;
    int v = 0;
    cudaMemcpy(&v, h->nn->derr, 4, cudaMemcpyDeviceToHost);
    return v;
}
void nn_destroy(ia_handle* h) {
    NNState* s = h->nn;
    if (!s) return;
    cudaFree(s->w); cudaFree(s->g); cudaFree(s->m); cudaFree(s->v);
    for (int l = 0; l < nn::NLAYER; ++l) cudaFree(s->wtc[l]);
    cudaFree(s->bias_tc); cudaFree(s->buf); cudaFree(s->ibuf); cudaFree(s->x16);
    cudaFree(s->dloss); cudaFree(s->derr); cudaFree(s->dscale);
    delete s;
    h->nn = nullptr;
}

}  // namespace ia

using namespace ia;

extern "C" {

int64_t ia_nn_param_count(void) { return nn::NPARAM; }

int ia_nn_set_params(ia_handle* h, const float* params) {
    if (!h || !params) return IA_ERR_INVALID;
    NNState* s = nn_state(h);
    if (!s) return IA_ERR_CUDA;
    if (cudaMemcpy(s->w, params, 4 * (size_t)nn::NPARAM, cudaMemcpyHostToDevice) != cudaSuccess) return IA_ERR_CUDA;
    cudaMemset(s->m, 0, 4 * (size_t)nn::NPARAM);
    cudaMemset(s->v, 0, 4 * (size_t)nn::NPARAM);
    s->step = 0;
    s->tc_dirty = true;
    return IA_OK;
}

int ia_nn_set_loss(ia_handle* h, int32_t kind) {
    if (!h || kind < 0 || kind > 1) return IA_ERR_INVALID;
    NNState* s = nn_state(h);
    if (!s) return IA_ERR_CUDA;
    s->loss_kind = kind;
    return IA_OK;
}

int ia_nn_get_params(ia_handle* h, float* params) {
    if (!h || !params) return IA_ERR_INVALID;
    NNState* s = nn_state(h);
    if (!s) return IA_ERR_CUDA;
    return cuda_fail(cudaMemcpy(params, s->w, 4 * (size_t)nn::NPARAM, cudaMemcpyDeviceToHost));
}

int ia_nn_forward(ia_handle* h, const float* x0, float* out, int32_t B, int32_t nx, int32_t ny, int32_t nz,
                  int32_t tensor_cores) {
    if (!h || !x0 || !out) return IA_ERR_INVALID;
    if (check_dims(B, nx, ny, nz) != IA_OK) return IA_ERR_INVALID;
    NNState* s = nn_state(h);
    if (!s) return IA_ERR_CUDA;
    const nn::Dims f{B, nx, ny, nz};
    cudaStream_t st = h->stream;
    if (!tensor_cores) {
        Graph G;
        if (ensure_graph(h, s, f, G) != IA_OK) return IA_ERR_CUDA;
        cudaMemcpyAsync(G.x0, x0, sizeof(float) * f.padded() * 4, cudaMemcpyDeviceToDevice, st);
        forward_f32(G, s->w, st);
        cudaMemcpyAsync(out, G.out, sizeof(float) * f.padded(), cudaMemcpyDeviceToDevice, st);
        return cuda_fail(cudaStreamSynchronize(st));
    }
    __nv_bfloat16* x16 = nullptr;
    if (cudaMalloc(&x16, 2 * 16 * (size_t)f.padded()) != cudaSuccess) return IA_ERR_CUDA;
    cudaMemsetAsync(x16, 0, 2 * 16 * (size_t)f.padded(), st);
    { nn::in_to_bf16<<<nblk(f.cells()), 256, 0, st>>>(f, x0, x16); ia::note_launch(); }
    cudaMemsetAsync(s->derr, 0, 4, st);
    int rc = forward_tc(h, s, f, x16, out);
    cudaError_t e = cudaStreamSynchronize(st);
    cudaFree(x16);
    if (rc != IA_OK || e != cudaSuccess) return IA_ERR_CUDA;
    return nn_error_flag(h) ? IA_ERR_CUDA : IA_OK;
}

int ia_nn_loss_grad(ia_handle* h, const float* x0, const float* target, int32_t B, int32_t nx, int32_t ny,
                    int32_t nz, float* grad, double* loss) {
    if (!h || !x0 || !target) return IA_ERR_INVALID;
    if (check_dims(B, nx, ny, nz) != IA_OK) return IA_ERR_INVALID;
    NNState* s = nn_state(h);
    if (!s) return IA_ERR_CUDA;
    int rc = loss_grad(h, s, x0, target, nn::Dims{B, nx, ny, nz}, loss);
    if (rc != IA_OK) return rc;
    if (grad) cudaMemcpyAsync(grad, s->g, 4 * (size_t)nn::NPARAM, cudaMemcpyDeviceToDevice, h->stream);
    return cuda_fail(cudaStreamSynchronize(h->stream));
}

int ia_nn_train_step(ia_handle* h, const float* x0, const float* target, int32_t B, int32_t nx, int32_t ny,
                     int32_t nz, float lr, double* loss) {
    if (!h || !x0 || !target) return IA_ERR_INVALID;
    if (check_dims(B, nx, ny, nz) != IA_OK) return IA_ERR_INVALID;
    NNState* s = nn_state(h);
    if (!s) return IA_ERR_CUDA;
    int rc = loss_grad(h, s, x0, target, nn::Dims{B, nx, ny, nz}, nullptr);
    if (rc != IA_OK) return rc;
    s->step += 1;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - std::pow(b1, float(s->step)), c2 = 1.f - std::pow(b2, float(s->step));
    { nn::adam_k<<<256, 256, 0, h->stream>>>(nn::NPARAM, s->w, s->g, s->m, s->v, lr, b1, b2, 1e-8f, c1, c2); ia::note_launch(); }
    s->tc_dirty = true;
    if (loss) {
        cudaMemcpyAsync(loss, s->dloss, 8, cudaMemcpyDeviceToHost, h->stream);
    }
    return cuda_fail(cudaStreamSynchronize(h->stream));
}

}  // extern "C"
