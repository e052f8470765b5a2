// Momentum, forcing and projection kernels of the two-phase step (mom.cu).
#pragma once
#include <cuda_runtime.h>

#include "ia_bc.cuh"
#include "ia_core.cuh"

namespace ia {

struct MomConsts {
    Grid g;
    double lrho, one_m, rho1, inv_lrho, inv_rho1;   // λρ, 1-λρ, λρ+(1-λρ)·1 and their reciprocals
    double uBC[3];
    double gvec[3];
    int has_g;
    int wide = 0;   // 1: the bulk passes' 64-bit offset variants whatever the grid size
};

// ρu2u! + BC! → uStar (src/VOFutil.jl:198-201; WaterLily BC!)
cudaError_t k_ustar(const MomConsts& k, const double* rhou, const double* f, double* ustar, cudaStream_t s);
// stage start: fd = fs, ud = us (when ud is given) on every cell, ρu = us·getρ(fs) on interior cells
cudaError_t k_stage_start(const MomConsts& k, const double* us, double* ud, const double* fs, double* fd, double* rhou,
                          cudaStream_t s);
// u2ρu! on interior cells (src/VOFutil.jl:208-211)
cudaError_t k_u2rhou(const MomConsts& k, double* rhou, const double* u, const double* f, cudaStream_t s);
// WaterLily BC! on a vector field in place
cudaError_t k_bc_vel(const MomConsts& k, double* a, const double* A, cudaStream_t s);
// CMOM face fluxes Φ_i at the lower j-faces (src/flow.jl:20-57, 212-241)
cudaError_t k_momflux(const MomConsts& k, int j, int limiter, const double* ustar, const double* rhouf_j,
                      const double* fold, double dt, double* Phi, cudaStream_t s);
// ρu += δt (Φ(I) - Φ(I+δj) + uOld ϕ(i,I,ρ̄∂ⱼuⱼ))
cudaError_t k_momupdate(const MomConsts& k, int j, const double* Phi, const double* uOld, const double* u1,
                        const double* u2, const int8_t* cbar, double dt, double* rhou, cudaStream_t s);
// visc! (src/flow.jl:119-153): symmetric face/edge fluxes then the divergence into r
cudaError_t k_visc(const MomConsts& k, const double* u, const double* f, double lmu, double mu, double* Phi6,
                   double* r, cudaStream_t s);
cudaError_t k_zero(double* a, long long n, cudaStream_t s);
// surfTen! (src/surfaceTension.jl:8-20) along every d: fb holds D face-fraction fields, list D cell
// lists of N entries, count D; prev0 (may be NULL = zeros) is the content of the reference's fbuffer
// before the call, of which only the high x-ghost plane is read
cudaError_t k_surften(const MomConsts& k, const double* f, const double* prev0, double eta, double* fb, double* r,
                      int* list, unsigned int* count, cudaStream_t s);
// updateU! (src/flow.jl:244-252) on interior cells; writes ρu when write_rhou
cudaError_t k_updateu(const MomConsts& k, double* u, double* rhou, const double* u0, const double* F, double dt,
                      const double* fref, const double* fupd, double w, bool write_rhou, cudaStream_t s);
// updateL! (src/flow.jl:254-259) incl. BC!(μ₀, 0)
cudaError_t k_updatel(const MomConsts& k, double* mu0, const double* f, cudaStream_t s);
// z = div(u) on interior cells, x *= dt (all cells)
cudaError_t k_div_scale(const MomConsts& k, const double* u, double* z, double* x, double dt, cudaStream_t s);
// u -= L ∂x (interior), x *= 1/dt (all), periodic ghosts of x
cudaError_t k_correct(const MomConsts& k, double* u, const double* L, double* x, double dt, cudaStream_t s);
// max flux_out and max maxTotalFlux over interior cells into out2 (device, as bit patterns)
cudaError_t k_cfl(const MomConsts& k, const double* u, unsigned long long* out2, cudaStream_t s);
// a *= f over n entries
cudaError_t k_scale(double* a, long long n, double f, cudaStream_t s);
// a = (a + b) / 2 over n entries
cudaError_t k_average(double* a, const double* b, long long n, cudaStream_t s);

// Float-float (FP32-pair) counterparts of the momentum chain (mom_ff.cu): uStar, the face fluxes and
// the viscous fluxes are pairs (float2); ρu, u and the forcing r stay FP64 fields.
cudaError_t k_ustar_ff(const MomConsts& k, const double* rhou, const double* f, float2* ustar, cudaStream_t s);
// k_stage_start plus the first sweep's uStar (the values k_ustar_ff gives after k_stage_start)
cudaError_t k_stage_start_ff(const MomConsts& k, const double* us, double* ud, const double* fs, double* fd, double* rhou,
                             float2* ustar, cudaStream_t s);
// uStar on the ghost cells only (some coordinate 0 or n-1), for a sweep whose interior cells k_momupdate_ff
// wrote
cudaError_t k_ustar_ff_planes(const MomConsts& k, const double* rhou, const double* f, float2* ustar,
                              cudaStream_t s);
// the bulk faces directly, every other cell through a list (list: N entries, count: one counter)
cudaError_t k_momflux_ff(const MomConsts& k, int j, int limiter, const float2* ustar, const double* rhouf_j,
                         const double* fold, double dt, float2* Phi, unsigned int* list, unsigned int* count,
                         int list_blocks, cudaStream_t s);
// dq: the dilation term ρ̄∂ⱼuⱼ/2 of every cell as pairs, written by the sweep's VOF bulk pass.  With
// us_next, also the next sweep's uStar from the new ρu and fn on the interior cells (the same values
// k_ustar_ff gives there)
cudaError_t k_momupdate_ff(const MomConsts& k, int j, const float2* Phi, const float2* dq, const double* uOld, double dt,
                           double* rhou, const double* fn, float2* us_next, cudaStream_t s);
cudaError_t k_visc_ff(const MomConsts& k, const double* u, const double* f, double lmu, double mu, float2* Phi6,
                      double* r, unsigned int* list, unsigned int* count, int list_blocks, cudaStream_t s);
// z = div(u) (pair sums), x *= dt; MPCFL's maxima with pair sums
cudaError_t k_div_scale_ff(const MomConsts& k, const double* u, double* zz, double* xx, double dt, cudaStream_t s);
cudaError_t k_cfl_ff(const MomConsts& k, const double* u, unsigned long long* out2, cudaStream_t s);
cudaError_t k_updateu_ff(const MomConsts& k, double* u, double* rhou, const double* u0, const double* F, double dt,
                         const double* fref, const double* fupd, double w, bool write_rhou, cudaStream_t s);

}  // namespace ia
