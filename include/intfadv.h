/*
 * libintfadv_gb300 — C-ABI of the GB300 (sm_103a) implementation of
 * InterfaceAdvection.jl's per-step hot path.
 *
 * Every entry point takes plain pointers and sizes.  Field arrays are DEVICE
 * pointers owned by the caller (Julia CuArrays, torch tensors, cudaMalloc),
 * laid out exactly as the reference's Julia arrays: column-major (x fastest),
 * one ghost layer (Ng = N + 2 per dimension), FP64, vector fields SoA with
 * the component index last (component d starts at d * prod(Ng)).  u[I,d] is
 * the velocity on the lower d-face of cell I.  Coordinates in this header are
 * 0-based (Julia index k is k-1).
 *
 * The library owns its scratch (ping-pong fraction buffers, interface-cell
 * lists, multigrid levels, status words) inside the handle.  All work is
 * ordered on the handle's CUDA stream; calls that report a status read it
 * back once per call.  Errors are return codes, never traps.
 *
 * Each entry point names the reference function it replaces
 * (file:line within the InterfaceAdvection.jl project).
 */
#ifndef INTFADV_H
#define INTFADV_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* ---- return codes ------------------------------------------------------- */
#define IA_OK                     0
#define IA_ERR_NAN                1   /* error("NaN!"), src/advection.jl:148           */
#define IA_ERR_DIVERGENCE         2   /* error("divergence ... exploding"), :160,:180  */
#define IA_ERR_UNSUPPORTED        3   /* udf, BDIM body, exitBC, D not in {2,3}, ...   */
#define IA_ERR_INVALID            4   /* bad argument / unbound field                  */
#define IA_ERR_CUDA               5   /* CUDA runtime error                            */
#define IA_ERR_NO_DEVICE          6
#define IA_ERR_TOO_LARGE          7   /* grid of 2^31 cells or more (ghosts included)  */
#define IA_WARN_FILL            100   /* over/under-fill past tol (printed, not fatal)  */
#define IA_WARN_NOT_CONVERGED   101   /* Poisson stopped at itmx                        */

/* status flag bits */
#define IA_FLAG_NAN        1u
#define IA_FLAG_OVERFILL   2u
#define IA_FLAG_UNDERFILL  4u
#define IA_FLAG_DIVERGENCE 8u
#define IA_FLAG_POISSON   16u

/* normalScheme (src/normalEstimation.jl) */
#define IA_NORMAL_WH      0   /* getInterfaceNormal_WH!  :105-154 (default) */
#define IA_NORMAL_WY      1   /* getInterfaceNormal_WY!  :35-68             */
#define IA_NORMAL_MYC     2   /* getInterfaceNormal_MYC! :185-202           */
#define IA_NORMAL_Y       3   /* getInterfaceNormal_Y!   :232-247           */
#define IA_NORMAL_COLUMN  4   /* getInterfaceNormal_Column! :75-97          */
#define IA_NORMAL_PCD     5   /* getInterfaceNormal_PCD! :161-165           */
#define IA_NORMAL_SLIC    6   /* getInterfaceNormal_SLIC! :172-176          */
#define IA_NORMAL_CD      7   /* getInterfaceNormal_CD!  :266-277           */
#define IA_NORMAL_XYLIC   8   /* getInterfaceNormal_XYLIC! :279-283         */

/* momentum-flux limiter λ(u,c,d) (src/flow.jl:5-15) */
#define IA_LIMITER_KOREN      0
#define IA_LIMITER_UPWIND     1
#define IA_LIMITER_MINMOD     2
#define IA_LIMITER_VANALBADA1 3
#define IA_LIMITER_SWEBY      4
#define IA_LIMITER_SUPERBEE   5
#define IA_LIMITER_TVDCEN     6
#define IA_LIMITER_TVDDOWN    7

/* Poisson solver modes */
#define IA_POISSON_FP64    0   /* FP64 V-cycle preconditioned CG                     */
#define IA_POISSON_MIXED   1   /* FP32 V-cycles inside FP64 defect-correction CG     */
#define IA_POISSON_LEARNED 2   /* as MIXED, inner FCG preconditioned by the conv net  */

/* Inner preconditioner of IA_POISSON_LEARNED (ia_poisson_precond) */
#define IA_PRECOND_HYBRID  0   /* s = Vcycle(r); s += ω·net(t), t = r - A s, ω energy-optimal */
#define IA_PRECOND_NET     1   /* s = net(r)                                           */
#define IA_PRECOND_NONE    2   /* s = r (plain CG; the ablation baseline)               */
#define IA_PRECOND_VCYCLE  3   /* s = Vcycle(r) (the fallback)                          */

/* Smoother of the FP32 V-cycle (ia_poisson_smoother) */
#define IA_SMOOTHER_HALFSWEEP 0   /* one launch per red-black half-sweep (the default)    */
#define IA_SMOOTHER_BLOCKED   1   /* all half-sweeps of a smoothing in one z-wavefront launch
                                     (3D); same arithmetic                                 */

/* Arithmetic of the momentum kernels (ia_momentum_arith) */
#define IA_ARITH_DEFAULT  (-1)  /* float-float in the MIXED / LEARNED modes, FP64 in the FP64 mode      */
#define IA_ARITH_FP64       0   /* FP64, as the reference computes (Float64 fields)                     */
#define IA_ARITH_FF         1   /* FP32 pairs (48-bit significands) built from error-free transformations */

typedef struct ia_handle ia_handle;

/* Construction parameters: TwoPhaseSimulation / cVOF keywords
 * (src/InterfaceAdvection.jl:67-84, src/cVOF.jl:45-89) plus the WaterLily
 * Flow settings the step reads (ν, constant g, constant u_BC, perdir). */
typedef struct {
    int32_t D;              /* 2 or 3 */
    int32_t perdir;         /* bit j set <=> dimension j (0-based) periodic */
    int64_t N[3];           /* interior cells per dimension (N[2] ignored for D=2) */
    double  lrho;           /* λρ = ρ_light / ρ_dark */
    double  lmu;            /* λμ = μ_light / μ_dark */
    double  mu;             /* dark-fluid dynamic viscosity; 0 = off (cVOF stores nothing) */
    double  eta;            /* surface tension coefficient; 0 = off */
    double  nu;             /* WaterLily ν (MPCFL advective limit) */
    double  g[3];           /* constant gravity; has_g = 0 => none */
    int32_t has_g;
    int32_t normal_scheme;  /* IA_NORMAL_* */
    int32_t limiter;        /* IA_LIMITER_* */
    int32_t poisson_mode;   /* IA_POISSON_* */
    double  uBC[3];         /* constant boundary velocity (WaterLily u_BC tuple) */
    double  poisson_tol;    /* L-infinity residual of the dt-scaled pressure system */
    int32_t poisson_itmx;
    int32_t exitBC;         /* must be 0: convective exit is not supported */
} ia_config;

/* Field pointers (device, FP64 unless noted), the reference's Flow and cVOF
 * members.  Pointers may be NULL for fields a call does not touch. */
typedef struct {
    /* WaterLily Flow */
    double *u, *u0, *force, *sigma, *p, *mu0;
    /* cVOF (src/cVOF.jl:1-44) */
    double *f, *f0, *alpha, *nhat, *fF, *rhou, *rhouf, *drho;
    int8_t *cbar;
} ia_fields;

/* Per-call status (one read-back per call). */
typedef struct {
    int32_t  code;              /* IA_OK, IA_ERR_*, IA_WARN_* (worst seen)        */
    uint32_t flags;             /* IA_FLAG_* */
    double   maxf, minf;        /* extreme fractions past tol (valid per flags)   */
    int64_t  maxid, minid;      /* their linear cell indices                      */
    int32_t  fill_dir;          /* 0-based sweep direction of the last flag       */
    int32_t  poisson_iters[2];  /* predictor / corrector solves                   */
    int32_t  pad;
    double   poisson_resid[2];  /* final L-infinity residuals (FP64)               */
    double   dt_next;           /* min(MPCFL, 1.2 dt) after ia_mom_step            */
} ia_status;

/* Create / destroy a solver handle.  Allocates the library's scratch on the
 * current device.  Replaces the allocation part of cVOF(N; ...) src/cVOF.jl:45-89
 * and TwoPhaseSimulation src/InterfaceAdvection.jl:67-84. */
int ia_create(const ia_config* cfg, ia_handle** out);
int ia_destroy(ia_handle* h);

/* Order all later work of this handle on `stream` (a cudaStream_t; NULL = legacy default). */
int ia_set_stream(ia_handle* h, void* stream);

/* Borrow the caller's field arrays (the Flow / cVOF members) for later calls. */
int ia_bind_fields(ia_handle* h, const ia_fields* fields);

/* advect!(a, c, f, u¹, u², dt) — src/advection.jl:17-23 → advectVOF! :34-78.
 * Lie–Trotter split VOF advection of `f` (in place) by the average of u1 and u2,
 * sweeping dimensions in the order dirO[i] = (n_dt + i) mod D, i = 1..D
 * (n_dt = length(Δt)).  Writes the bound c̄ and, if bound, ρuf. */
int ia_advect_vof(ia_handle* h, double* f, const double* u1, const double* u2,
                  double dt, int64_t n_dt, ia_status* status);

/* Allocation-free variant of ia_advect_vof for callers that cannot let a
 * library allocate device memory at run time (frameworks that reserve the
 * device memory up front for their own pool, time-stepping loops that forbid
 * the device-wide synchronisation of cudaMalloc/cudaFree after set-up).  It has
 * no counterpart in the reference.  It needs no handle: the caller passes the
 * configuration, a cudaStream_t (NULL = legacy default), the fields (f updated
 * in place, c̄ written, ρuf written when not NULL) and gets the same results as
 * ia_advect_vof.  Its scratch is one fixed-size device array inside the library
 * (24 MiB + 1 KiB, held by every GPU that loads the library until exit):
 * grids above IA_NOALLOC_MAX_CELLS ghost-inclusive cells return
 * IA_ERR_TOO_LARGE; every call reuses the array (status and counters are
 * cleared at the start of each call), so calls whose GPU work overlaps race and
 * must be serialised by the caller.  The array is per device: `stream` must
 * belong to the current device (IA_ERR_INVALID otherwise), and the first call
 * on a device looks up the array's address there.  Like ia_advect_vof, the
 * call reads its status back and synchronises `stream` before returning, so it
 * must not be called inside a stream capture.  exitBC is rejected with
 * IA_ERR_UNSUPPORTED, as by ia_create. */
#define IA_NOALLOC_MAX_CELLS 1048576
int ia_advect_vof_noalloc(const ia_config* cfg, void* stream, double* f, const double* u1,
                          const double* u2, double dt, int64_t n_dt, int8_t* cbar, double* rhouf,
                          ia_status* status);

/* reconstructInterface!(f, α, n̂, normalScheme) — src/normalEstimation.jl:10-28,
 * including BCVOF! src/VOFutil.jl:44-55 (f ghosts updated in place). */
int ia_reconstruct(ia_handle* h, double* f, double* alpha, double* nhat);

/* getVOFFlux!(fᶠ, f, α, n̂, u, u⁰, δt, d, ρuf, λρ) — src/advection.jl:108-137
 * (fᶠ zeroed first; ρuf[:,d] accumulated when rhouf is not NULL). */
int ia_vof_flux(ia_handle* h, double* fF, const double* f, const double* alpha,
                const double* nhat, const double* u, const double* u0, double dt,
                int32_t d, double* rhouf);

/* applyVOF!(f, α, n̂, SDF) + BCf! — src/VOFutil.jl:9-37, src/cVOF.jl:56.
 * `sdf` holds 1 + 2D scalar fields: the SDF at cell centres, then at
 * centre ± 0.01 e_d for d = 0..D-1 (+ first).  Interior cells only. */
int ia_apply_vof(ia_handle* h, const double* sdf, double* f, double* alpha, double* nhat);

/* MPFMomStep!(flow, pois, intf, body; δt) — src/flow.jl:60-109, the body of
 * sim_step!(::TwoPhaseSimulation) src/InterfaceAdvection.jl:100-103.
 * Density-weighted RK2 step on the bound fields: CMOM momentum advection fused
 * with the VOF sweeps (split order from n_dt = length(Δt)), viscous and
 * surface-tension forcing, velocity update with constant gravity, projection
 * (poisson_mode, poisson_tol, poisson_itmx of the config), then
 * status->dt_next = min(MPCFL, 1.2 dt) for push!(Δt, ·).  `dt` is δt = last(Δt).
 * Required bound fields: u, u0, force, sigma, p, mu0, f, f0, rhou, rhouf. */
int ia_mom_step(ia_handle* h, double dt, int64_t n_dt, double t_now, ia_status* status);

/* MPCFL(flow, intf) — src/flow.jl:262-281 (on the bound u). */
int ia_cfl(ia_handle* h, double* dt_out);

/* WaterLily BC!(a, u_BC, false, perdir) on a vector field, as the reference
 * calls it on u, ρu, ρuf and μ₀ (src/flow.jl:69,79,82,207,258). */
int ia_bc_velocity(ia_handle* h, double* a);

/* Pressure solve of inproject!(::MultiLevelPoisson) — src/flow.jl:343-347
 * (WaterLily solver!): A x = z with the face coefficients L (μ₀), x holding the
 * initial guess; stops when the L-infinity FP64 residual is <= tol or after itmx
 * iterations (IA_WARN_NOT_CONVERGED). */
int ia_poisson_solve(ia_handle* h, double* x, const double* z, const double* L, double tol,
                     int32_t itmx, int32_t* iters, double* resid);

/* Residual of that pressure system, r = z - A x on interior cells, and its L-infinity norm
 * (the quantity ia_poisson_solve's stopping test measures; src/flow.jl:343-347). */
int ia_poisson_residual(ia_handle* h, double* r, const double* x, const double* z, const double* L,
                        double* linf);

/* updateL!(μ₀, f) + myproject!(flow, pois, w) — src/flow.jl:254-259, 328-347, with
 * dtp = w·last(Δt), on the bound u, p, sigma (source) and mu0; then BC!(u). */
int ia_project(ia_handle* h, const double* f, double dtp, int32_t* iters, double* resid);

/* advectfq!(flow, intf, f, u¹, u², uOld, δt) — src/flow.jl:157-232: momentum
 * advection of the bound ρu fused with the VOF advection of f. */
int ia_advect_momentum(ia_handle* h, double* f, const double* u1, const double* u2,
                       const double* uOld, double dt, int64_t n_dt, ia_status* status);

/* Arithmetic of the momentum chain of ia_mom_step / ia_advect_momentum / ia_visc_surften (uStar,
 * the CMOM face fluxes, the momentum update, the viscous fluxes, updateU!): IA_ARITH_FP64,
 * IA_ARITH_FF or IA_ARITH_DEFAULT.  No reference counterpart: the reference computes in the field
 * type T.  The float-float path keeps every FP64 field and the FP64 VOF, PLIC, Poisson defect
 * correction and rare mixed-cell branches; only the momentum arithmetic runs on FP32 pairs
 * (relative precision about 2^-46 per operation), because GB300 issues FP64 at 1/64 of the FP32 rate. */
int ia_momentum_arith(ia_handle* h, int32_t kind);

/* viscSurfTenρu!(r, u, ...) — src/flow.jl:113-117 into the bound force field,
 * with the fraction f (the reference's f⁰ midpoint or f). */
int ia_visc_surften(ia_handle* h, const double* f);

/* surfTen!(forcing, f, α, n̂, fbuffer, η) — src/surfaceTension.jl:8-20: for every direction d
 * the face fraction ϕ(d,·,f) with BCf!(d, ·), the WY normal and the Popinet height-function
 * curvature on the cells whose face fraction is mixed, forcing[I,d] += η κ (−∂(d,I,f)).
 * `forcing` is a device vector field (accumulated into), `f` the fraction.  The reference reuses
 * fbuffer (the cVOF's fᶠ) for every d, and BCf!(d, ·) never writes its high ghost along a wall
 * dimension d, so that position holds the buffer's previous content; `fbuffer` supplies that content
 * for d = 1 (its high x-ghost plane is read, nothing is written to it; NULL = zeros, which is what
 * fᶠ holds there after a VOF sweep between walls of zero normal velocity).  η = 0 is η::Nothing (no-op). */
int ia_surften(ia_handle* h, double* forcing, const double* f, const double* fbuffer, double eta);

/* Σ f over interior cells (FP64, deterministic tree order): the mass the
 * reference checks with sum(f[inside(f)]), test/maintests.jl:209,215. */
int ia_mass(ia_handle* h, const double* f, double* mass_out);

/* Level-set reinitialisation (src/redistaning.jl).  Buffers are caller-owned scalar fields
 * (the reference reuses f⁰ for ϕ, α for ϕ⁰, fᶠ for ϕ_ini and σ for L).
 * ia_levelset_init: ϕ = 2f - 1 and ϕ_ini = ϕ on every cell (LevelSet, :13-25; phi_ini may be NULL).
 * ia_levelset_rhs:  L = ϕ_ini (1 - |∇ϕ|) with ENO2 one-sided derivatives (computeL!, :64-143).
 * ia_redistance:    round(d/dτ) SSP-RK3 pseudo-time steps of ∂τϕ = L(ϕ) with BCf! ghosts after
 *                   each stage (redistaning!, :42-54). */
int ia_levelset_init(ia_handle* h, const double* f, double* phi, double* phi_ini);
int ia_levelset_rhs(ia_handle* h, double* L, const double* phi, const double* phi_ini);
int ia_redistance(ia_handle* h, double* phi, double* phi0, const double* phi_ini, double* L, double d,
                  double dtau);

/* Step diagnostics of src/metrics.jl summed over interior cells, in one pass:
 * out[0] = Σ ρkeI(I,u,f,λρ,U) (:13-15), out[1] = Σ ρgh(I,g,f,λρ,StatWL) (:23),
 * out[2] = Σ EnsI(I,ω) (:32-39; 0 when omega is NULL), out[3+i] = Σ ρuI(i,I,u,f,λρ,U) (:56-58).
 * omega: 3D vector field (component i on the edges the reference's EnsI reads), 2D scalar.
 * U, g, statwl: D values each, NULL = zeros. */
int ia_metrics(ia_handle* h, const double* u, const double* f, const double* omega, const double* U,
               const double* g, const double* statwl, double* out);

/* Per-launch kernel timing with CUDA events on the handle's stream, for the
 * roofline figures (no reference counterpart: instrumentation only).
 * Folds finished records into per-family totals, copies the first n totals
 * (milliseconds, launch counts; families: 0 VOF bulk sweep, 1 VOF list sweep,
 * 2 momentum sweep, 3 forcing/update, 4 MG V-cycle, 5 MG residual,
 * 6 MG transfer, 7 Krylov vector ops, 8 other, 9 VOF faces, 10 momentum flux,
 * 11 momentum update, 12 update/projection, 13 finest-level red-black
 * half-sweeps, 14 learned preconditioner, 15 finest-level first half-sweeps),
 * then, if enable >= 0, resets the totals and switches recording on (1) or
 * off (0). */
int ia_timing(ia_handle* h, int32_t enable, double* ms_out, int64_t* launches_out, int32_t n);

/* Measured FMA throughput of the current device, FP64 and FP32, in fused multiply-adds per second
 * per device (instrumentation for the roofline figures; no reference counterpart). */
int ia_probe_fma_rates(double* fp64_fma_per_s, double* fp32_fma_per_s);

/* Number of CUDA kernels this library has launched in the process so far
 * (instrumentation, no reference counterpart; used for launch accounting). */
int64_t ia_launch_count(void);

const char* ia_error_string(int code);

/* ---------------------------------------------------------------------------
 * Learned Poisson preconditioner (no reference counterpart).
 *
 * Network: 3-level 3D conv encoder-decoder, 3x3x3 kernels, channels
 * 4-16-32-32-32-16-1 (see csrc/nn.cuh), input channels r/max|r| and λρ·L_{x,y,z},
 * output ∝ A⁻¹ r.  Parameters: FP32 vector of ia_nn_param_count() floats, per
 * layer W[27][Cout][Cin] (tap = (dz+1)*9 + (dy+1)*3 + (dx+1)) then b[Cout].
 * Training tensors (device, FP32): channels-last with a one-cell zero halo,
 * x0 [B][nz+2][ny+2][nx+2][4], target and out [B][nz+2][ny+2][nx+2];
 * nx, ny, nz multiples of 4.  A handle of any grid carries the net state.
 * ------------------------------------------------------------------------- */
int64_t ia_nn_param_count(void);
/* copy host parameters into / out of the handle's net (set resets the Adam moments) */
int ia_nn_set_params(ia_handle* h, const float* params);
int ia_nn_get_params(ia_handle* h, float* params);
/* forward pass on the handle's stream: tensor_cores = 0 FP32 training kernels, 1 the BF16
 * tcgen05 inference kernels fed by TMA row windows (the solver's path) */
int ia_nn_forward(ia_handle* h, const float* x0, float* out, int32_t B, int32_t nx, int32_t ny, int32_t nz,
                  int32_t tensor_cores);
/* training loss (mean over interior cells) and its gradient (device, NULL = keep in the handle) */
int ia_nn_loss_grad(ia_handle* h, const float* x0, const float* target, int32_t B, int32_t nx, int32_t ny,
                    int32_t nz, float* grad, double* loss);
/* training loss of the handle's net: 0 = mean squared error (default), 1 = energy norm of the
 * error, Σ_cells Σ_d c_d (δ[p] - δ[p-e_d])² / n with c_d the input coefficient channels */
int ia_nn_set_loss(ia_handle* h, int32_t kind);
/* one Adam step (β1 0.9, β2 0.999, ε 1e-8) on the training loss of the handle's net; loss before
 * the step */
int ia_nn_train_step(ia_handle* h, const float* x0, const float* target, int32_t B, int32_t nx, int32_t ny,
                     int32_t nz, float lr, double* loss);
/* inner preconditioner of an IA_POISSON_LEARNED handle and the inner FCG limits
 * (inner_max iterations, relative inner residual target); an IA_POISSON_MIXED handle accepts
 * IA_PRECOND_VCYCLE only (to set its inner limits) */
int ia_poisson_precond(ia_handle* h, int32_t precond, int32_t inner_max, double inner_rtol);
/* V-cycle smoothing of the handle's multigrid (no reference counterpart; the reference's
 * MultiLevelPoisson settings are WaterLily's): nu1 red-black sweeps before and nu2 after the
 * coarse correction, nuc symmetric sweeps on the coarsest level (defaults 2, 2, 16) */
int ia_poisson_mg_params(ia_handle* h, int32_t nu1, int32_t nu2, int32_t nuc);
/* smoother of the FP32 V-cycle (no reference counterpart: the reference smooths in FP64 with
 * WaterLily's MultiLevelPoisson): IA_SMOOTHER_*.  The blocked smoother is used where it applies
 * (3D levels, nu1 and nu2 in {1, 2}, relaxation factor 1) and the half-sweeps elsewhere */
int ia_poisson_smoother(ia_handle* h, int32_t kind);
/* relaxation factor omega in (0, 2) of the V-cycle's red-black half-sweeps, x += omega (x_GS - x)
 * (no reference counterpart; default 1.15, which takes the rising-bubble solves from 12 to 10 FCG
 * iterations per step; 1 is plain Gauss-Seidel); the coarsest-level sweeps stay at 1.  The blocked
 * smoother runs only at omega = 1 (the half-sweeps are used otherwise) */
int ia_poisson_mg_relax(ia_handle* h, double omega);
/* coefficient storage of the finest level's V-cycle smoother in the MIXED / LEARNED modes (no reference
 * counterpart): 1 = an FP16 copy of the FP32 face coefficients (relative precision 2^-11) for the
 * red-black half-sweeps and the residual restriction of that level, 0 = the FP32 coefficients.  The inner
 * FCG's operator, the coarse levels and the FP64 defect correction are not affected, so the solve still
 * stops on the FP64 true residual.  Default 1 when the coefficients 1/ρ (between 1/max(λρ,1) and
 * 1/min(λρ,1)) fit FP16's range, which IA_ERR_UNSUPPORTED reports otherwise. */
int ia_poisson_coef16(ia_handle* h, int32_t on);
/* 1: the momentum and viscous flux bulk passes use their 64-bit cell-offset variants whatever the grid
 * size; 0 (default): the 32-bit variants wherever every vector entry index fits 32 bits (fewer
 * instructions per address), the 64-bit ones beyond.  Same results either way; the switch lets the
 * 64-bit variants be tested on small grids (no reference counterpart). */
int ia_wide_offsets(ia_handle* h, int32_t on);
/* smoothings of the finest level's half-sweep V-cycle (no reference counterpart): nu1 pre- and nu2
 * post-smoothings on the finest level only, the coarser levels keeping ia_poisson_mg_params' counts;
 * 0 = the same as the coarser levels (default).  nu1 >= 1 takes effect; 0..16. */
int ia_poisson_mg_fine(ia_handle* h, int32_t nu1, int32_t nu2);
/* rows per slab of the finest-level wavefront in the MIXED / LEARNED modes (no reference counterpart):
 * the red-black half-sweeps and the residual restriction of a smoothing run slab by slab over y, each
 * half-sweep one row behind the previous, so that the later half-sweeps read the slab from L2.  Same
 * results as whole-level half-sweeps, bit for bit.  0 = whole-level half-sweeps; otherwise at least 8.
 * Applies in 3D with walls in y.  Default 0: with two z planes per half-sweep thread the wavefront no
 * longer shortens the step (a slab within about 3/5 of L2, 64 rows at 256x512x256, ties). */
int ia_poisson_slab_rows(ia_handle* h, int32_t rows);
/* counters since the handle's creation: [0] net applications, [1] V-cycles, [2] fallbacks
 * to the V-cycle, [3] inner FCG iterations, [4] outer corrections */
int ia_poisson_stats(ia_handle* h, int64_t* out5);

#ifdef __cplusplus
}
#endif
#endif
