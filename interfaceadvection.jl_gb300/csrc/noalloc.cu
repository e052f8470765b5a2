// ia_advect_vof_noalloc: advect! without any allocation by the library.
//
// Some callers cannot let a library allocate device memory at run time:
// host frameworks that reserve (nearly) all device memory up front for their
// own pool (so a raw cudaMalloc from a third-party library fails or fragments
// their pool), and time-stepping loops that forbid allocation once set up
// because cudaMalloc/cudaFree synchronise the device and stall the stream.
// They still own and pass the fields; this entry point needs no handle and
// takes its scratch (interface-cell and face lists, cached face fluxes,
// staged values, the status block) from one file-scope device array of fixed
// size, which every GPU that loads the library holds until the process exits.
//
// Limits and sharing rules:
//  * grids up to IA_NOALLOC_MAX_CELLS ghost-inclusive cells; larger grids are
//    rejected with IA_ERR_TOO_LARGE before any GPU work;
//  * every call uses the same array and it keeps the previous call's
//    contents: the status block and list counters are cleared at the start of
//    each call; calls whose GPU work overlaps (other streams, other host
//    threads) race on the array and must be serialised by the caller;
//  * the array is per device: `stream` must belong to the current device
//    (checked; IA_ERR_INVALID otherwise).  The first call on a device looks up
//    the array's device address with cudaGetSymbolAddress (that device
//    current) and caches it;
//  * the call ends with a status read-back and a synchronisation of `stream`
//    (like ia_advect_vof), so it cannot be made inside a stream capture.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>

#include "../../include/intfadv.h"
#include "capi_internal.cuh"
#include "ia_core.cuh"
#include "vof.cuh"

namespace {

constexpr size_t kMaxCells = (size_t)IA_NOALLOC_MAX_CELLS;
constexpr size_t kStatusBytes = 1024;   // DevStatus, rounded up to keep the lists 256-byte aligned
constexpr size_t kListBytes = 4 * kMaxCells;
constexpr size_t kFluxBytes = 8 * kMaxCells;
constexpr size_t kScratchBytes = kStatusBytes + 2 * kListBytes + 2 * kFluxBytes;
static_assert(sizeof(ia::DevStatus) <= kStatusBytes, "status block must fit its slot");

// the only scratch of ia_advect_vof_noalloc (24 MiB + 1 KiB)
static __device__ __align__(256) unsigned char ia_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
static void* g_scratch_dev[kMaxDevices];   // device address per device ordinal, set on first use

__global__ void noalloc_reset_k(ia::DevStatus* s) {
    s->flags = 0;
    s->dir = 0;
    s->max_enc = 0ull;
    s->min_enc = ~0ull;
    s->max_key = 0ull;
    s->min_key = 0ull;
    for (int i = 0; i < 32; ++i) s->list_count[i] = 0;
}

int scratch_address(void** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return IA_ERR_NO_DEVICE;
    if (!g_scratch_dev[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, ia_noalloc_scratch) != cudaSuccess || !p) return IA_ERR_CUDA;
        g_scratch_dev[dev] = p;
    }
    *out = g_scratch_dev[dev];
    return IA_OK;
}

}  // namespace

extern "C" int ia_advect_vof_noalloc(const ia_config* cfg, void* stream, double* f, const double* u1,
                                     const double* u2, double dt, int64_t n_dt, int8_t* cbar, double* rhouf,
                                     ia_status* status) {
    if (!cfg || !f || !u1 || !u2 || !cbar) return IA_ERR_INVALID;
    if (cfg->D != 2 && cfg->D != 3) return IA_ERR_UNSUPPORTED;
    if (cfg->exitBC) return IA_ERR_UNSUPPORTED;   // as ia_create
    if (cfg->normal_scheme < 0 || cfg->normal_scheme > IA_NORMAL_XYLIC) return IA_ERR_INVALID;
    for (int d = 0; d < cfg->D; ++d)
        if (cfg->N[d] < 2) return IA_ERR_INVALID;
    const ia::Grid g = ia::make_grid(cfg->D, cfg->perdir, cfg->N);
    if ((size_t)g.N > kMaxCells) return IA_ERR_TOO_LARGE;
    void* base = nullptr;
    int rc = scratch_address(&base);
    if (rc != IA_OK) return rc;
    unsigned char* b = static_cast<unsigned char*>(base);
    ia::DevStatus* dst = reinterpret_cast<ia::DevStatus*>(b);
    unsigned int* list = reinterpret_cast<unsigned int*>(b + kStatusBytes);
    unsigned int* flist = reinterpret_cast<unsigned int*>(b + kStatusBytes + kListBytes);
    double* flux = reinterpret_cast<double*>(b + kStatusBytes + 2 * kListBytes);
    double* vals = reinterpret_cast<double*>(b + kStatusBytes + 2 * kListBytes + kFluxBytes);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int sms = 152, dev = 0, sdev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return IA_ERR_NO_DEVICE;
    // the scratch address above is the current device's: a stream of another device would run
    // the kernels against that device's copy of nothing this call prepared
    if (cudaStreamGetDevice(st, &sdev) != cudaSuccess || sdev != dev) return IA_ERR_INVALID;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int list_blocks = sms * 8;

    noalloc_reset_k<<<1, 1, 0, st>>>(dst);
    if (cudaGetLastError() != cudaSuccess) return IA_ERR_CUDA;
    const double tol = 10.0 * 2.220446049250313e-16;
    double lim = (dt > 0.0 && std::isfinite(dt)) ? 0.5 / dt : 0.0;
    for (int k = 0; k < g.D; ++k) {
        ia::SweepArgs a;
        a.g = g;
        a.d = int((n_dt + k + 1) % g.D);   // dirO, src/advection.jl:22
        a.scheme = cfg->normal_scheme;
        a.first = (k == 0);
        a.fin = f;
        a.fout = f;
        a.u1 = u1 + (long long)a.d * g.N;
        a.u2 = u2 + (long long)a.d * g.N;
        a.cbar = cbar;
        a.rhouf_d = rhouf ? rhouf + (long long)a.d * g.N : nullptr;
        a.h = dt / 2.0;
        a.dt = dt;
        a.lrho = cfg->lrho;
        a.one_m_lrho = 1.0 - cfg->lrho;
        a.hl = (dt / 2.0) * cfg->lrho;
        a.tol_rep = tol;
        a.tol_clean = tol;
        std::memcpy(&a.ulim, &lim, 8);
        a.list = list;
        a.list_count = &dst->list_count[2 * k];
        a.flist = flist;
        a.flist_count = &dst->list_count[2 * k + 1];
        a.flux = flux;
        a.vals = vals;
        a.st = dst;
        if (ia::vof_sweep_bulk(a, st) != cudaSuccess) return IA_ERR_CUDA;
        if (ia::vof_sweep_faces(a, st, list_blocks) != cudaSuccess) return IA_ERR_CUDA;
        if (ia::vof_sweep_cells(a, st, list_blocks) != cudaSuccess) return IA_ERR_CUDA;
        if (ia::vof_sweep_scatter(a, st, list_blocks) != cudaSuccess) return IA_ERR_CUDA;
    }
    // one status read-back into host stack memory (pageable: no pinned allocation)
    ia::DevStatus hs;
    if (cudaMemcpyAsync(&hs, dst, sizeof(hs), cudaMemcpyDeviceToHost, st) != cudaSuccess) return IA_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return IA_ERR_CUDA;
    ia_status s;
    std::memset(&s, 0, sizeof(s));
    const int code = ia::translate_fill_status(g, hs, u1, u2, s);
    if (status) *status = s;
    return code;
}
