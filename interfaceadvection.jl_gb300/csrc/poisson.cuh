// Multigrid hierarchy and Krylov state of the pressure solve (poisson.cu).
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "ia_core.cuh"

struct ia_handle;

namespace ia {

constexpr int MG_MAX_LEVELS = 12;

// Step scalars of the mixed solver's inner FCG, kept on the device so that only the convergence test
// is read back each iteration: β and α in FP64 (and as the FP32 values the vector kernels use), the
// previous step's α and s·r, the stop flag of a breakdown, and L∞ of the inner residual (FP32 bits).
struct FcgDev {
    double alpha_prev, rho_prev, sr, beta;
    float beta32, alpha32;
    unsigned int rin;   // read back together with stop (8 bytes)
    int stop;
    unsigned int done_dot, done_mv;   // blocks finished in the current reduction kernel (0 between launches)
};

struct MGLevel {
    Grid g;
    // FP64 operator and vectors (IA_POISSON_FP64)
    double *x = nullptr, *b = nullptr, *r = nullptr, *L = nullptr, *iD = nullptr;
    // FP32 operator and vectors (IA_POISSON_MIXED)
    float *x32 = nullptr, *b32 = nullptr, *r32 = nullptr, *L32 = nullptr, *iD32 = nullptr;
    // finest level of the mixed V-cycle: FP16 copy of L32 for the smoother and the residual restriction
    __half* L16 = nullptr;
    template <class T> T* x_();
    template <class T> T* b_();
    template <class T> T* r_();
    template <class T> T* L_();
    template <class T> T* iD_();
};
template <> inline double* MGLevel::x_<double>() { return x; }
template <> inline double* MGLevel::b_<double>() { return b; }
template <> inline double* MGLevel::r_<double>() { return r; }
template <> inline double* MGLevel::L_<double>() { return L; }
template <> inline double* MGLevel::iD_<double>() { return iD; }
template <> inline float* MGLevel::x_<float>() { return x32; }
template <> inline float* MGLevel::b_<float>() { return b32; }
template <> inline float* MGLevel::r_<float>() { return r32; }
template <> inline float* MGLevel::L_<float>() { return L32; }
template <> inline float* MGLevel::iD_<float>() { return iD32; }

}  // namespace ia

struct PoissonMG {
    int nlev = 0;
    ia::MGLevel lev[ia::MG_MAX_LEVELS];
    double *r = nullptr, *s = nullptr, *p = nullptr, *q = nullptr;   // fine-level Krylov vectors (FP64)
    float *p32 = nullptr, *q32 = nullptr, *e32 = nullptr;             // inner FP32 Krylov vectors (mixed)
    float *rl32 = nullptr, *nl32 = nullptr, *t32 = nullptr;           // learned: residual, net output, A·net
    int precond = 0;                                                  // IA_PRECOND_* of the learned mode
    long long stats[5] = {0, 0, 0, 0, 0};                             // net, V-cycles, fallbacks, inner, outer
    int inner_max = 30;                                               // inner FCG iterations per correction
    double inner_rtol = 1e-3;                                         // inner relative residual target
    double* partial = nullptr;                                        // per-block dot partials
    long long mvb = 0;                                                // blocks (partials) of the tiled FP32 matvec
    int kb = 0;                                                       // blocks of the Krylov row loops
    double* diag64 = nullptr;                                         // FP64 operator diagonal
    double* dsc = nullptr;                                            // device scalars
    ia::FcgDev* fcg = nullptr;                                        // the inner FCG's step scalars
    double* hsc = nullptr;                                            // pinned host scalars
    int nu1 = 2, nu2 = 2, nuc = 16;
    int nu1f = 0, nu2f = 0;                                           // finest-level smoothings (0: nu1, nu2)
    int smoother = 0;                                                 // IA_SMOOTHER_* (FP32 V-cycle)
    double omega = 1.15;                                              // smoother relaxation factor
    int coef16 = 0;                                                   // finest-level smoother on L16 (mixed)
    int slab_rows = 0;                                                // finest-level wavefront slab (rows; 0 off)
    int nsm = 0;                                                      // multiprocessors of the device
    // each precision's finest-level V-cycle is captured once into a CUDA graph (its launch
    // sequence and arguments are fixed for the handle) and replayed; recaptured when the
    // smoothing parameters change
    cudaGraphExec_t vgraph[2] = {nullptr, nullptr};   // FP32, FP64
    long long vgraph_kernels[2] = {0, 0};
    int vgraph_nu[2][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}};
    double vgraph_omega[2] = {1.0, 1.0};
    int vgraph_c16[2] = {0, 0};
    int vgraph_slab[2] = {0, 0};
    int vgraph_fine[2] = {0, 0};                                      // nu1f * 64 + nu2f of the graph
    cudaStream_t capture = nullptr;
};

namespace ia {
int mg_create(ia_handle* h);
bool coef16_fits(double lrho);
void mg_destroy(ia_handle* h);
int poisson_solve(ia_handle* h, double* x, const double* z, const double* L, double tol, int itmx, int* iters,
                  double* resid);
int poisson_residual(ia_handle* h, double* r, const double* x, const double* z, const double* L, double* linf);
}  // namespace ia
