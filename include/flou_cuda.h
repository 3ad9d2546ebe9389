/*
 * flou_cuda.h -- C ABI of libflou_cuda, the GB300 (sm_103a) FP64 implementation of Flou.jl's
 * DGSEM semidiscrete residual and its explicit Runge-Kutta stepping.
 *
 * Every entry point is `extern "C"`, takes plain pointers and sizes, and returns an int32
 * status (FLOU_OK = 0).  flou_last_error(ctx) gives a message for the last failure on ctx.
 *
 * Conventions (those of Flou's own containers, so a Julia caller passes its arrays as is):
 *   - The state is a column-major (ndofs_total x nvars) Float64 matrix: each variable is one
 *     contiguous column; element e (1-based) owns rows (e-1)*n^d+1 .. e*n^d; element nodes are
 *     ordered i fastest (src/FlouSpatial/GlobalContainers.jl:19-50, DofHandler.jl:62-68,
 *     StdRegions/StdRegions.jl:60-62).
 *   - Square operator matrices are n x n column-major (Julia Matrix{Float64}).
 *   - Mesh connectivity uses the reference's 1-based indices (src/FlouCommon/Mesh.jl:26-133).
 *   - Pointers to state arrays may be host or device memory, chosen by `ptr_kind`.
 *
 * Threading: a context is used by one host thread at a time; distinct contexts may be used
 * concurrently.  Each context launches on one CUDA stream (its own, or the caller's after
 * flou_set_stream).
 */
#ifndef FLOU_CUDA_H
#define FLOU_CUDA_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------------- */
#define FLOU_OK 0
#define FLOU_ERR_ARG 1          /* invalid argument or inconsistent sizes                  */
#define FLOU_ERR_CUDA 2         /* a CUDA runtime call failed                                */
#define FLOU_ERR_NONPHYSICAL 3  /* rho <= 0, p <= 0 or a non-finite value was produced       */
#define FLOU_ERR_TIMEOUT 4      /* a bounded device-side wait ran out                        */
#define FLOU_ERR_OOM 5          /* device allocation failed                                   */
#define FLOU_ERR_UNSUPPORTED 6  /* valid in Flou but outside this library                      */
#define FLOU_ERR_STATE 7        /* call order violated (e.g. rhs before set_mesh)            */
#define FLOU_ERR_INDEX 8        /* a device index check failed (FLOU_CUDA_CHECKED builds only) */

/* ---- enumerations --------------------------------------------------------------------- */
/* Equations: LinearAdvection (src/FlouCommon/LinearAdvection.jl:16-26), BurgersEquation
 * (src/FlouCommon/Burgers.jl:16), EulerEquation{ND}(γ) (src/FlouCommon/Euler.jl:16-24). */
#define FLOU_EQ_LINEAR_ADVECTION 0
#define FLOU_EQ_BURGERS 1
#define FLOU_EQ_EULER 2

/* Volume operators: StrongDivOperator (OpDivergence.jl:105-160; weak == strong on LGL),
 * SplitDivOperator (OpDivergence.jl:184-437; on a basis without boundary nodes the entropy-
 * projected form of :301-437, Euler only). */
#define FLOU_OP_STRONG 0
#define FLOU_OP_SPLIT 1
/* HybridDivOperator (OpDivergence.jl:439-801): the split form in telescopic (subcell) form,
 * blended with a subcell finite-volume flux; Euler.  The FV flux and the blending constant are
 * set with flou_set_hybrid; general (non-Cartesian) geometry also needs flou_set_subgrid. */
#define FLOU_OP_HYBRID 2

/* Two-point volume fluxes of the split form: StdAverage (Euler.jl:385-472),
 * ChandrasekharAverage (Euler.jl:474-536), Kennedy-Gruber (no Flou counterpart). */
#define FLOU_TP_STD_AVERAGE 0
#define FLOU_TP_CHANDRASHEKAR 1
#define FLOU_TP_KENNEDY_GRUBER 2

/* Interface (numerical) fluxes: StdAverage (Euler.jl:99-136), LxF(avg, intensity) =
 * Rusanov (Euler.jl:138-165), ChandrasekharAverage (Euler.jl:167-226), HLL and HLLC (no Flou
 * counterpart; Toro's formulation with Davis wave speeds). */
#define FLOU_NF_STD_AVERAGE 0
#define FLOU_NF_LXF 1
#define FLOU_NF_CHANDRASHEKAR 2
#define FLOU_NF_HLL 3
#define FLOU_NF_HLLC 4
/* Entropy-stable dissipation added to a central flux (numflux_avg: StdAverage or
 * ChandrasekharAverage), Euler only: ScalarDissipation (Euler.jl:228-301) and
 * MatrixDissipation (Euler.jl:303-380). */
#define FLOU_NF_SCALAR_DISSIPATION 5
#define FLOU_NF_MATRIX_DISSIPATION 6

/* Boundary conditions applied on boundary faces (periodic faces are interior faces after
 * apply_periodicBCs!): EulerOutflowBC, EulerInflowBC(Qext), EulerSlipBC
 * (src/FlouSpatial/Equations/Euler.jl:69-94).  Inflow/outflow also serve the scalar
 * equations (a constant Dirichlet state / zero-gradient copy). */
#define FLOU_BC_OUTFLOW 1
#define FLOU_BC_INFLOW 2
#define FLOU_BC_SLIP 3
/* A Dirichlet state given per boundary face node (a GenericBC whose Qext(x) varies along the
 * boundary, FlouSpatial.jl:80-91), set with flou_set_bc_field. */
#define FLOU_BC_STATE_FIELD 4

/* Pointer kinds for state arrays. */
#define FLOU_PTR_HOST 0
#define FLOU_PTR_DEVICE 1

typedef struct flou_ctx flou_ctx;

/* Replaces the set-up of EquationConfig(MultielementDisc(mesh, std, equation, operator,
 * bcs), equation) (src/FlouCommon/FlouCommon.jl:92-95,
 * src/FlouSpatial/MultielementDiscontinuous.jl:29-92). */
typedef struct flou_config {
    int32_t dim;               /* 1, 2 or 3                                                 */
    int32_t equation;          /* FLOU_EQ_*                                                 */
    double gamma;              /* EulerEquation γ                                           */
    double advection[3];       /* LinearAdvection velocity (unused entries 0)               */
    int32_t volume_op;         /* FLOU_OP_*                                                 */
    int32_t twopoint_flux;     /* FLOU_TP_* (split form only)                               */
    int32_t numflux;           /* FLOU_NF_*                                                 */
    int32_t numflux_avg;       /* central flux inside LxF and the dissipation fluxes:
                                  FLOU_NF_STD_AVERAGE or FLOU_NF_CHANDRASHEKAR                  */
    double numflux_intensity;  /* LxF intensity (1.0 = Rusanov)                             */
    int32_t nnodes;            /* nodes per direction n = p + 1, 2 <= n <= 8                */
} flou_config;

/* ---- context lifecycle ------------------------------------------------------------------ */
int32_t flou_create(const flou_config* cfg, flou_ctx** out);
int32_t flou_destroy(flou_ctx* ctx);
const char* flou_last_error(const flou_ctx* ctx);
/* Launch on the caller's stream (a cudaStream_t); NULL restores the context's own stream. */
int32_t flou_set_stream(flou_ctx* ctx, void* stream);

/* ---- set-up uploads (deep copies; the caller keeps ownership) -------------------------- */
/* Std-region operators of StdSegment (src/FlouSpatial/StdRegions/StdSegment.jl:77-89):
 * D, Ds = D - B, D♯ = 2D - B (n x n), ω, l_l, l_r, ∂g_l, ∂g_r (n).  StdQuad/StdHex reuse the
 * segment's matrices (StdQuad.jl:61-67, StdHex.jl:79-85). */
int32_t flou_set_operators(flou_ctx* ctx, const double* D, const double* Ds, const double* Dsharp,
                           const double* omega, const double* l_l, const double* l_r, const double* dg_l,
                           const double* dg_r);

/* Connectivity of the mesh after apply_periodicBCs! (src/FlouCommon/Mesh.jl:236-322):
 *   faceinds/facepos: nelem x 2d, element-major (mesh.elements[e].faceinds/.facepos);
 *   eleminds/elempos: nfaces x 2 (mesh.faces[f].eleminds/.elempos), eleminds[.,2] = 0 on
 *   boundary faces; orientation: nfaces (mesh.faces[f].orientation);
 *   bdface_index: nfaces, the boundary index (1-based, position in mesh.bdfaces) of each
 *   boundary face, 0 for interior faces. */
int32_t flou_set_mesh(flou_ctx* ctx, int32_t nelem, int32_t nfaces, const int32_t* faceinds, const int32_t* facepos,
                      const int32_t* eleminds, const int32_t* elempos, const uint8_t* orientation,
                      const int32_t* bdface_index);

/* Boundary conditions per boundary index (MultielementDisc's _bcs tuple,
 * MultielementDiscontinuous.jl:40-51): kinds[nbcs] (FLOU_BC_*), states[nbcs x 5]
 * (the Qext of inflow conditions, row per boundary). */
int32_t flou_set_bcs(flou_ctx* ctx, int32_t nbcs, const int32_t* kinds, const double* states);
/* External states of the FLOU_BC_STATE_FIELD boundaries: states[nfaces x n^(dim-1) x 5], the face
 * nodes in the face-dof order of each face (master side), 5 values per node (zero-padded); the
 * entries of other faces are not read. */
int32_t flou_set_bc_field(flou_ctx* ctx, const double* states);

/* Geometry (Geometry, src/FlouSpatial/PhysicalRegions.jl:982-991): per node J (ndofs),
 * metric Ja (ndofs x d x d, column-major per node); per face node the frame
 * (nfacedofs x 3 x 3: n, t, b with 3 components each) and the surface Jacobian
 * (nfacedofs).  Cartesian geometry (J and a diagonal Ja constant per element, the Cartesian
 * frames, every face orientation 0) takes a compressed fast path; any other geometry
 * (curvilinear / unstructured, PhysicalRegions.jl:438-472 and :756-971) is used per node, in 2D
 * or 3D.  Rejected: J <= 0, non-finite entries, non-unit normals, surface Jacobians <= 0. */
int32_t flou_set_geometry(flou_ctx* ctx, const double* J, const double* Ja, const double* frames,
                          const double* face_J);

/* The hybrid operator's subcell finite-volume flux (HybridDivOperator's fvflux: FLOU_NF_* with
 * its central flux and intensity) and blending constant c (δ = max((√(b²+c) - b)/√(b²+c), 1/2),
 * OpDivergence.jl:777-801).  Required before the first residual of a FLOU_OP_HYBRID context. */
int32_t flou_set_hybrid(flou_ctx* ctx, int32_t fvflux, int32_t fvflux_avg, double fvflux_intensity, double blend);
/* Subcell-interface geometry of general (curvilinear / unstructured) elements, which the hybrid
 * operator's subcell finite-volume fluxes and, on a basis without boundary nodes, the split
 * form's projected states need (geometry.subgrids, PhysicalRegions.jl:180-300):
 * for element e, direction d, line m (the face-dof order of a face normal to d) and interface
 * s = 0..n of that line, point ((e·dim + d)·n^(dim-1) + m)·(n+1) + s holds the unit normal, tangent
 * and binormal (9 doubles in `frames`, zero-padded to 3 components) and the surface Jacobian
 * (`jac`).  Required before stepping such a context whose geometry is not Cartesian. */
int32_t flou_set_subgrid(flou_ctx* ctx, const double* frames, const double* jac);

/* ---- residual and stepping ------------------------------------------------------------- */
/* FlouCommon.rhs!(dQ, Q, p::EquationConfig{<:MultielementDisc,<:HyperbolicEquation}, t)
 * (src/FlouSpatial/Equations/Hyperbolic.jl:31-69): dQ is overwritten.  Synchronous. */
int32_t flou_rhs(flou_ctx* ctx, double* dQ, const double* Q, double t, int32_t ptr_kind);

/* `nsteps` Shu-Osher SSP-RK3 steps of size dt (or steps of the method of flou_set_integrator), in
 * place on Q (the SSPRK33 solver that timeintegrate hands to OrdinaryDiffEq,
 * src/FlouTime/FlouTime.jl:34-54).  Each stage's
 * combination is fused into the residual kernel; the step is replayed as a CUDA graph.
 * Returns FLOU_ERR_NONPHYSICAL when any stage produced rho <= 0, p <= 0 or a non-finite
 * value (Flou raises a DomainError there, FlouTime.jl:37-51). */
int32_t flou_step(flou_ctx* ctx, double* Q, double dt, double t0, int32_t nsteps, int32_t ptr_kind);

/* The step method of flou_step / flou_step_async.  nstages = 0 restores the Shu-Osher SSP-RK3
 * (the default).  nstages in 1..FLOU_MAX_LSRK_STAGES selects the 2N-storage Runge-Kutta method
 * (Williamson 1980) with coefficients A[0..s-1] (A[0] is not read) and B[0..s-1]:
 *   k = dt L(u); u += B[0] k;   for i = 1..s-1: k = A[i] k + dt L(u); u += B[i] k,
 * the LowStorageRK2N form of OrdinaryDiffEq 6.49.1 with williamson_condition = false, which
 * the reference steps its tests and examples with (ORK256, test/tests.jl:19,56,93,139;
 * CarpenterKennedy2N54).  No boundary condition on this path depends on time, so the stage
 * abscissae are not needed.  Each stage is one residual whose element epilogue updates k and
 * u in place; the limiter, when set, acts after every stage.  The adjoint and the batched
 * launch step with SSP-RK3 only. */
#define FLOU_MAX_LSRK_STAGES 16

/* CFL-limited stepping: get_cfl_callback(cfl, dtmax) (src/FlouTime/FlouTime.jl:92-105) with the
 * step method of flou_set_integrator.  Before every step dt = min(get_max_dt(Q, cfl), dtmax), and
 * the last step is cut to land on tfinal (OrdinaryDiffEq stops on tfinal).  The time, dt and the
 * step count live on the device: each step is one CUDA graph (CFL bound, step control, stages),
 * the host only reads the state back between batches of steps.  Stops after max_steps steps at
 * most; *nsteps receives the steps taken, *t_out the time reached (tfinal unless max_steps cut
 * the run short).  dtmax may be +inf.  The limiter and the monitors act as in flou_step.
 * FLOU_ERR_NONPHYSICAL when a state breaks or no positive time step exists. */
int32_t flou_step_cfl(flou_ctx* ctx, double* Q, double t0, double tfinal, double cfl, double dtmax,
                      int64_t max_steps, int32_t ptr_kind, int64_t* nsteps, double* t_out);
int32_t flou_set_integrator(flou_ctx* ctx, int32_t nstages, const double* A, const double* B);

/* flou_step without the final synchronisation: the copies (host pointers; use pinned memory
 * for them to overlap) and the steps are queued on the context's stream and the call returns.
 * The state must stay untouched until flou_wait(ctx), which synchronises and reports the status
 * (FLOU_ERR_NONPHYSICAL as flou_step would).  Contexts on different streams overlap one
 * another's copies and kernels.  No counterpart in the reference. */
int32_t flou_step_async(flou_ctx* ctx, double* Q, double dt, double t0, int32_t nsteps, int32_t ptr_kind);
int32_t flou_wait(flou_ctx* ctx);

/* get_max_dt(q, disc, eq, cfl) (src/FlouSpatial/MultielementDiscontinuous.jl:162-178). */
int32_t flou_max_dt(flou_ctx* ctx, const double* Q, double cfl, double* dt, int32_t ptr_kind);

/* The residual of flou_rhs without any device allocation: device pointers only, face
 * fluxes kept in a fixed 8 MiB array inside the library (at most 1,048,576 values of
 * nfaces x n^(d-1) x nvars), shared by all calls, so overlapping calls race.  For callers
 * whose device memory belongs to another allocator (CUDA.jl's pool, PyTorch's caching
 * allocator), where flou_rhs's lazy cudaMalloc of its face buffer could fail or is not
 * allowed.  It accepts exactly the contexts flou_rhs accepts (FLOU_ERR_STATE, before any
 * launch, when a set-up call the operator needs is missing).  The first call on a device
 * looks up the array's address and caches it for the process; make it before any stream
 * capture, and make no call on a device after cudaDeviceReset.  No counterpart in the
 * reference. */
int32_t flou_rhs_noalloc(flou_ctx* ctx, double* dQ, const double* Q, double t);

/* Number of nodes (DOFs in Flou's sense, DofHandler.jl:53) and of variables. */
int32_t flou_sizes(const flou_ctx* ctx, int64_t* ndofs, int32_t* nvars, int32_t* nelem, int32_t* nfaces);

/* Status word of the last device work on ctx: bit 0 = non-physical state seen; *elem = the
 * lowest element index (1-based) that raised it, 0 if none.  Clears the word. */
int32_t flou_take_status(flou_ctx* ctx, int32_t* flags, int32_t* elem);

/* Times the two kernels of one RK stage on the context's stream with CUDA events: `nrep`
 * launches of the face kernel and of the element kernel in each of the three stage modes
 * (Q is a device state; the results go to internal scratch).  Returns the mean duration of
 * one launch in milliseconds.  No counterpart in the reference (measurement hook). */
int32_t flou_time_kernels(flou_ctx* ctx, const double* Q, int32_t nrep, double* face_ms, double* elem_ms);

/* Host-only validation (no GPU needed) of the set-up arrays exactly as flou_set_mesh /
 * flou_set_geometry check them; msg receives the reason (may be NULL).  No counterpart in the
 * reference (Flou's constructors build these arrays themselves). */
int32_t flou_check_mesh(int32_t dim, int32_t nelem, int32_t nfaces, const int32_t* faceinds, const int32_t* facepos,
                        const int32_t* eleminds, const int32_t* elempos, const uint8_t* orientation,
                        const int32_t* bdface_index, char* msg, int32_t msglen);
int32_t flou_check_geometry(int32_t dim, int32_t nnodes, int32_t nelem, int32_t nfaces, const int32_t* elempos,
                            const double* omega, const double* J, const double* Ja, const double* frames,
                            const double* face_J, char* msg, int32_t msglen);

/* Measured FP64 fused-multiply-add throughput of the current device in GFLOP/s (2 flops per
 * FMA), used as the FP64 roofline denominator.  No counterpart in the reference. */
int32_t flou_fp64_peak(double* gflops);
/* The same for the FP64 tensor cores: m8n8k4 DMMA (mma.sync with f64 operands) throughput in
 * GFLOP/s, the measurement behind the choice of CUDA-core FP64 for the derivative-matrix
 * contraction.  No counterpart in the reference. */
int32_t flou_fp64_dmma_peak(double* gflops);
/* Accuracy check of the FP64 reciprocal and square root the kernels build from the MUFU
 * approximations refined by one third-order step: the largest error against the correctly rounded
 * 1/x and sqrt(x) over nsamples doubles with exponents in [2^-40, 2^40], in units of 2^-53
 * relative (2 = 1 ulp).  No counterpart in the reference. */
int32_t flou_check_refined_math(int64_t nsamples, double* rcp_err, double* sqrt_err);

/* ---- discrete adjoint (no counterpart in the reference; Flou differentiates nothing) ----
 * Covers linear advection (1D-3D, Cartesian or general geometry) and Burgers (1D) with the strong
 * form (either node set) or the split form with the StdAverage two-point flux, the LxF or
 * StdAverage interface flux; and the Euler equations with
 *  - the strong form, the split form (Chandrashekar, Kennedy-Gruber or StdAverage two-point
 *    flux) and the hybrid operator (any interface flux below as its subcell flux);
 *  - the LxF, ScalarDissipation or MatrixDissipation interface flux (StdAverage or
 *    ChandrasekharAverage central part), HLL and HLLC;
 *  - Gauss-Lobatto or Gauss nodes, Cartesian or general geometry;
 *  - periodic, slip-wall, outflow, inflow and boundary-state-field boundaries (fixed external
 *    states are constants of the differentiation);
 *  - SSP-RK3 or the 2N-storage method set by flou_set_integrator, with or without the Zhang-Shu
 *    stage limiter (in flou_adjoint_solve_batch each instance with its own);
 *  - every order p = 1..7.
 * Other contexts return FLOU_ERR_UNSUPPORTED.
 * Non-smooth points follow Julia's Base (ForwardDiff on the reference's CPU path):
 * max(a, b) takes b unless b < a; d|u|/du = -1 for a set sign bit, else +1. */

/* Per-element scale c_e of the LxF dissipation: a face uses intensity (c_1 + c_2)/2 of its
 * two elements (c_1 on boundary faces); c = 1 everywhere reproduces LxF(StdAverage(), 1.0).
 * NULL removes it.  c has nelem entries (host or device memory by ptr_kind). */
int32_t flou_set_dissipation(flou_ctx* ctx, const double* c, int32_t ptr_kind);

/* Vector-Jacobian product of the residual at Q (device pointers):
 * Qbar = (∂rhs/∂Q)ᵀ lambda, cbar = (∂rhs/∂c)ᵀ lambda (cbar may be NULL; needs the scale c). */
int32_t flou_rhs_vjp(flou_ctx* ctx, double* Qbar, double* cbar, const double* Q, const double* lambda);

/* Gradient of J = 1/2 Σ_i w_i (ρ_i(T) - ρt_i)², T = nsteps·dt, with respect to the initial state
 * Q0 and the dissipation scales c, by the discrete adjoint of the SSP-RK3 solve with binomial
 * checkpointing: at most `nsnap` stored states besides Q0 (the schedule minimising recomputed
 * forward steps for that budget).  Device pointers: Q0, rho_target, weights (ndofs), dJdQ0
 * (state-sized), dJdc (nelem, may be NULL).  *forward_steps (may be NULL) returns the number of
 * recomputed forward steps. */
int32_t flou_adjoint_solve(flou_ctx* ctx, const double* Q0, double dt, int32_t nsteps, int32_t nsnap,
                           const double* rho_target, const double* weights, double* J, double* dJdQ0, double* dJdc,
                           int64_t* forward_steps);

/* Gradients of n independent solves (same functional form, same number of steps, each its own
 * dt, context and targets) in one lockstep reverse sweep under one device-memory budget: one
 * checkpoint schedule serves every instance, a snapshot holds all their states at one step,
 * and the number of snapshots is what `budget_bytes` leaves after the step scratch (the
 * schedule minimising recomputed forward steps for it).  The instances' kernels run on
 * `nstreams` internal streams (<= 0: 8), the largest instances spread across them.
 * Device pointers per instance: Q0[k] (read only; it is snapshot 0), rho_target[k] and
 * weights[k] (ndofs), dJdQ0[k] (state-sized), dJdc[k] (nelem; dJdc or dJdc[k] may be NULL).
 * Host outputs: J[k] (may be NULL), *forward_steps (recomputed forward steps per instance)
 * and *nsnap (snapshots used); either may be NULL.  On failure every context's last error
 * names the instance.  No counterpart in the reference. */
int32_t flou_adjoint_solve_batch(int32_t n, flou_ctx* const* ctxs, double* const* Q0, const double* dt,
                                 int32_t nsteps, int64_t budget_bytes, int32_t nstreams,
                                 double* const* rho_target, double* const* weights, double* J,
                                 double* const* dJdQ0, double* const* dJdc, int64_t* forward_steps,
                                 int32_t* nsnap);

/* ---- stage limiter and integral monitors (Euler) ----------------------------------------------
 * The Zhang-Shu positivity limiter of src/FlouSpatial/Equations/Euler.jl:611-654 (`get_limiter`
 * :zhang_shu with its minimum value), applied after every stage of flou_step /
 * flou_step_async / flou_step_cfl, as Flou's `get_limiter_callback` passed as OrdinaryDiffEq's stage_limiter!
 * (src/FlouTime/FlouTime.jl:136-148).  Per element: the density, then all variables, are scaled
 * toward the element mean when the minimum density / pressure falls below min(minval, mean). */
#define FLOU_LIMITER_NONE 0
#define FLOU_LIMITER_ZHANG_SHU 1
int32_t flou_set_limiter(flou_ctx* ctx, int32_t kind, double minval);
/* The set limiter applied once to Q in place (host or device memory by ptr_kind). */
int32_t flou_limit(flou_ctx* ctx, double* Q, int32_t ptr_kind);
/* Integral monitors (Euler.jl:541-590, get_monitor :energy / :entropy): Σ_e Jω'·f(Q) with f the
 * kinetic energy |ρv|²/(2ρ) or the mathematical entropy -ρ(log p - γ log ρ)/(γ-1). */
#define FLOU_MONITOR_KINETIC_ENERGY 1
#define FLOU_MONITOR_ENTROPY 2
int32_t flou_monitor(flou_ctx* ctx, const double* Q, int32_t which, double* value, int32_t ptr_kind);
/* Monitors recorded after every step of flou_step / flou_step_async (Flou's
 * get_monitor_callback with iter=true) into a device buffer of `capacity` steps, without host
 * synchronisation; mask = OR of FLOU_MONITOR_* bits (0 stops recording).  flou_take_monitors
 * copies the values recorded since the last take, two per step (kinetic energy, entropy;
 * unselected ones are 0), and restarts the record; FLOU_ERR_STATE if more steps ran than
 * `capacity`. */
int32_t flou_set_monitors(flou_ctx* ctx, int32_t mask, int32_t capacity);
int32_t flou_take_monitors(flou_ctx* ctx, double* out, int32_t max_steps, int32_t* nsteps);
/* flou_take_monitors plus the time after each recorded step (flou_step_cfl; NaN for steps of
 * flou_step, whose times t0 + k dt the caller knows). */
int32_t flou_take_monitors_timed(flou_ctx* ctx, double* out, double* times, int32_t max_steps, int32_t* nsteps);

/* ---- batched mode (no counterpart in the reference: Flou solves one problem at a time) ----
 * Many independent discretizations with uneven element counts and orders advance together:
 * one persistent launch per stage serves every instance from one work queue of face items and
 * element tiles, and the stages of a step replay as one CUDA graph.  A batch is built from
 * contexts whose set-up is complete; they must outlive the batch and share the dimension,
 * equation and volume operator (2D Euler strong form, or 3D Euler split form with the
 * Chandrashekar flux), the time integrator (SSP-RK3, or one 2N-storage method for all) and the
 * kind of geometry (all Cartesian or all general); an instance with the Zhang-Shu limiter gets
 * it after every stage, one with monitors records them after every step.  States are device
 * pointers, one per instance. */
typedef struct flou_batch flou_batch;
int32_t flou_batch_create(int32_t n, flou_ctx* const* ctxs, flou_batch** out);
int32_t flou_batch_destroy(flou_batch* b);
const char* flou_batch_last_error(const flou_batch* b);
int32_t flou_batch_set_stream(flou_batch* b, void* stream);
/* Q[k]: device state of instance k (advanced in place); dt[k]: its fixed time step. */
int32_t flou_batch_set_states(flou_batch* b, double* const* Q, const double* dt);
/* nsteps steps of every instance.  FLOU_ERR_TIMEOUT if a bounded device-side wait ran
 * out (the results of that call are then invalid; the batch stays usable). */
int32_t flou_batch_step(flou_batch* b, int32_t nsteps);
/* Autotuner: times the first stage for every (threads per block, resident blocks per SM,
 * element-item order) candidate and keeps the fastest; out = {threads, blocks/SM, order}. */
int32_t flou_batch_autotune(flou_batch* b, int32_t* out);
/* Element tiles per work item the autotuner chose for each order (tiles[n - 2] for n = 2..8 nodes
 * per direction; 1 before tuning).  No counterpart in the reference. */
int32_t flou_batch_tiles(const flou_batch* b, int32_t* tiles);
/* Sets those tiles per work item (1..8 for each of the 7 orders) instead of tuning them.  No
 * counterpart in the reference. */
int32_t flou_batch_set_tiles(flou_batch* b, const int32_t* tiles);
/* Fault-injection hook for tests: instance `inst`'s face items never report completion, so its
 * element tiles run out of their bounded wait; -1 restores normal operation. */
int32_t flou_batch_test_skip_faces(flou_batch* b, int32_t inst);

#ifdef __cplusplus
}
#endif

#endif /* FLOU_CUDA_H */
