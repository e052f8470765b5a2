// Handle layout and helpers shared by the C-ABI translation units.
#pragma once
#include <cuda_runtime.h>

#include "ia_core.cuh"
#include "vof.cuh"

#include <vector>

// Kernel families timed by the optional per-launch event instrumentation.
enum TimedKernel { TK_VOF_BULK = 0, TK_VOF_LIST = 1, TK_MOM = 2, TK_FORCE = 3, TK_MG_SMOOTH = 4,
                   TK_MG_RESID = 5, TK_MG_TRANSFER = 6, TK_KRYLOV = 7, TK_OTHER = 8, TK_VOF_FACES = 9,
                   TK_MOM_FLUX = 10, TK_MOM_UPDATE = 11, TK_UPDATE = 12, TK_MG_FINE = 13, TK_NN = 14, TK_MG_FIRST = 15,
                   TK_COUNT = 16 };

struct Timing {
    bool on = false;
    std::vector<cudaEvent_t> pool;     // reusable events
    std::vector<int> fam;              // family of record k (events 2k, 2k+1)
    size_t used = 0;
    double ms[TK_COUNT] = {0};
    long long launches[TK_COUNT] = {0};
};

struct MomScratch;    // momentum / projection scratch (momentum.cu)
struct PoissonMG;     // multigrid hierarchy (poisson.cu)
namespace ia { struct NNState; }   // learned preconditioner: weights, Adam state, buffers (nn.cu)

struct ia_handle {
    ia_config cfg;
    ia::Grid g;
    int device;
    int list_blocks;
    cudaStream_t stream;
    ia_fields fld;
    // scratch owned by the library
    double* tmp1 = nullptr;            // staged values of listed cells
    unsigned int* list = nullptr;      // compacted cells needing the full update
    unsigned int* flist = nullptr;     // compacted faces needing reconstruction
    double* flux = nullptr;            // cached fluxes of listed faces
    ia::DevStatus* dst = nullptr;      // device status
    ia::DevStatus* hst = nullptr;      // pinned host mirror
    double* partial = nullptr;         // reduction partials
    double* dscalar = nullptr;         // device scalars
    int8_t* cbar_own = nullptr;        // c̄ when the caller binds none
    int mom_arith = -1;                // IA_ARITH_* of the momentum kernels (-1: by Poisson mode)
    int wide_offsets = 0;              // ia_wide_offsets
    Timing timing;
    MomScratch* mom = nullptr;
    PoissonMG* mg = nullptr;
    ia::NNState* nn = nullptr;
};

namespace ia {
int cuda_fail(cudaError_t e);
int status_reset(ia_handle* h);
int status_collect(ia_handle* h, const double* u1, const double* u2, ia_status* out, bool merge);
// Host-side translation of one read-back device status into `st` (flags OR-ed in, fill extremes,
// the divergence check of both velocity fields at a flagged cell) and the reportFillError return
// code (src/advection.jl:145-189).  Shared by every entry point that reports a fill status.
int translate_fill_status(const Grid& g, const DevStatus& s, const double* u1, const double* u2, ia_status& st);
// one VOF sweep along d, fin -> fout (fin == fout: in place); dila (coupled momentum step, float-float
// arithmetic): receives the momentum update's dilation term of every cell as FP32 pairs
int vof_sweep(ia_handle* h, const double* fin, double* fout, const double* u1, const double* u2, double dt, int d,
              bool first, int8_t* cbar, double* rhouf, double tol_rep, int counter, float2* dila = nullptr);
int advect_sweeps(ia_handle* h, double* f, const double* u1, const double* u2, double dt, const int* dirs,
                  int nsweeps, int8_t* cbar, double* rhouf, double tol_rep, bool first_writes_cbar,
                  int counter_base);
// allocation hooks of the momentum / Poisson modules
// per-launch timing: begin returns a token (-1 when off); end closes it
int timing_begin(ia_handle* h, int family);
void timing_end(ia_handle* h, int token);
int extra_create(ia_handle* h);
void extra_destroy(ia_handle* h);
// learned preconditioner (nn.cu): out = net(r / max|r|, λρ·L) on a 3D grid, interior written
int nn_apply(ia_handle* h, const float* r, const float* L32, float* out, int nx, int ny, int nz, long long ncomp);
int nn_error_flag(ia_handle* h);
void nn_destroy(ia_handle* h);
}  // namespace ia
