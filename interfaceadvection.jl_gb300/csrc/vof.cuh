// VOF sweep launcher interface (see vof.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "ia_core.cuh"

namespace ia {

struct SweepArgs {
    Grid g;
    int d;                            // sweep direction (0-based)
    int scheme;                       // IA_NORMAL_*
    bool first;                       // first sweep of the call: computes and writes c̄
    const double* fin;                // fractions before the sweep (ghosts valid)
    double* fout;                     // fractions after the sweep: the same array (in place)
    const double* __restrict__ u1;    // component d of the first velocity field
    const double* __restrict__ u2;    // component d of the second velocity field
    int8_t* cbar;                     // c̄: written when first, read otherwise
    double* rhouf_d;                  // component d of ρuf (written in full), or nullptr
    double h;                         // δt / 2
    double dt;                        // δt of the sweep
    double lrho;                      // λρ
    double one_m_lrho;                // 1 - λρ
    double hl;                        // δt/2 · λρ
    double tol_rep;                   // reportFillError tolerance
    double tol_clean;                 // cleanWisp! tolerance (10 eps)
    unsigned long long ulim;          // bit pattern of 1/(2δt): fast-path velocity bound
    unsigned int* list;               // cells needing the full update
    unsigned int* list_count;
    unsigned int* flist;              // faces whose donor needs reconstruction
    unsigned int* flist_count;
    double* flux;                     // cached face fluxes of listed faces
    double* vals;                     // staged new values of listed cells
    DevStatus* st;
    // coupled momentum step only (NULL otherwise): d = getρ(I,c̄,λρ)(∂(d,I,u1) + ∂(d,I,u2))/4 of every cell
    // (ghosts from their boundary-condition source cell) as FP32 pairs (hi, lo), the dilation term the
    // momentum update reads (src/flow.jl:216, 229); rq = λρ/4 and (λρ + (1-λρ))/4 as pairs
    float2* dila = nullptr;
    float rq_l_hi = 0.f, rq_l_lo = 0.f, rq_1_hi = 0.f, rq_1_lo = 0.f;
};

cudaError_t vof_sweep_bulk(const SweepArgs& a, cudaStream_t st);
cudaError_t vof_sweep_faces(const SweepArgs& a, cudaStream_t st, int list_blocks);
cudaError_t vof_sweep_cells(const SweepArgs& a, cudaStream_t st, int list_blocks);
cudaError_t vof_sweep_scatter(const SweepArgs& a, cudaStream_t st, int list_blocks);

// applyVOF! interior + BCf! ghosts
cudaError_t apply_vof(const Grid& g, const double* sdf, double* f, double* alpha, double* nhat, cudaStream_t st);
// reconstructInterface! + BCVOF!
cudaError_t reconstruct(const Grid& g, int scheme, double* f, double* alpha, double* nhat, cudaStream_t st);
// getVOFFlux! with caller-supplied α, n̂
cudaError_t vof_flux(const Grid& g, double* fF, const double* f, const double* alpha, const double* nhat,
                     const double* u, const double* u0, double dt, int d, double* rhouf, double lrho,
                     cudaStream_t st);
// ghosts of a scalar from their boundary-condition source cells (BCf!)
cudaError_t fill_ghosts_scalar(const Grid& g, double* f, cudaStream_t st);
// deterministic Σ over interior cells; partial buffer of >= 4096 doubles
cudaError_t interior_sum(const Grid& g, const double* f, double* partial, double* out, cudaStream_t st);

}  // namespace ia
