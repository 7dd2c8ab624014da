/* hc.h -- C ABI of the GB300 residual-and-timestep path.
 *
 * One context owns one 2D structured mesh, its boundary conditions, a solution
 * state and the device buffers of an explicit Runge-Kutta integrator.  All
 * calls are synchronous unless named *_async; none throws; every function
 * returns an hc_status and hc_last_error_string() describes the last failure
 * of the calling thread.  A context is not thread-safe; distinct contexts are
 * independent.  Arrays are plain host pointers unless the name ends in _device.
 *
 * The reference (lacrymose/hyperboliConvergence, header-only C++20) has no ABI;
 * each entry point below replaces the C++ interface named beside it.
 *
 * Array layouts: cell (i,j) of an ni x nj mesh is element i*nj + j; state
 * arrays are 4 planes of ni*nj values; node arrays hold (ni+1)*(nj+1) points
 * as x,y pairs, node (i,j) at 2*(i*(nj+1)+j).
 */
#ifndef HC_H
#define HC_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct hc_ctx hc_ctx;

typedef enum {
  HC_OK = 0,
  HC_ERR_ARG = 1,         /* invalid argument or call order */
  HC_ERR_CUDA = 2,        /* CUDA runtime failure */
  HC_ERR_NONPHYSICAL = 3, /* a step produced rho<=0, p<=0 or a non-finite value */
  HC_ERR_TIMEOUT = 4,     /* a bounded device wait gave up */
  HC_ERR_UNSUPPORTED = 5  /* combination not built */
} hc_status;

/* Interface flux (FluxFunctor, conservationLaws/base/concepts.h:97-107) */
typedef enum {
  HC_FLUX_ROE = 0,      /* RoeFlux<Euler>, conservationLaws/base/fluxes/roeFlux.ipp:2-58 */
  HC_FLUX_SLAU = 1,     /* SLAU2 upwinded by the sign of the mass flux */
  HC_FLUX_SLAU_REF = 2, /* Slau<Convective,Acoustic> as written, conservationLaws/euler/fluxes/slau.ipp:4-161 */
  HC_FLUX_AUSMPUP = 3,  /* AusmPlusUP<V,P>, conservationLaws/euler/fluxes/ausmPlusUP.ipp:6-171;
                           (Convective,Convective) unless hc_set_low_mach chooses V and P */
  HC_FLUX_RUSANOV = 4,  /* RusanovFlux<Euler>, conservationLaws/base/fluxes/rusanovFlux.ipp:2-50 */
  HC_FLUX_CENTRAL = 5,  /* CentralFlux<Euler>, conservationLaws/base/fluxes/centralFlux.ipp:2-14 */
  HC_FLUX_ROE_WS = 6,   /* RoeUnprecWS, conservationLaws/euler/fluxes/roeUnprecWS.ipp:2-109 */
  HC_FLUX_ROE_FACE = 7  /* RoeFlux with the Roe-averaged velocity taken into the face frame of the
                           jump: RoeDissipation (roeFlux.ipp:40-54) rotates the jump but not the
                           averaged state, so HC_FLUX_ROE is the Roe matrix's dissipation only for
                           the face normal (1, 0); this variant is rotation-invariant and equal to
                           HC_FLUX_ROE bit for bit for that normal.  Not in the reference. */
} hc_flux;

/* LowMachScaling (conservationLaws/euler/euler.h:331-339): AUSM+up's velocity (V) and
 * pressure (P) diffusion scalings */
typedef enum { HC_SCALING_CONVECTIVE = 0, HC_SCALING_ACOUSTIC = 1, HC_SCALING_ADAPTIVE = 2 } hc_scaling;

/* Slope limiter (VariableLimiterInterface, limiters/limiter.h:14-28) */
typedef enum {
  HC_LIM_NOLIMIT1 = 0, HC_LIM_NOLIMIT2 = 1, HC_LIM_NOLIMIT3 = 2, HC_LIM_VANALBADA = 3,
  HC_LIM_MINMOD = 4, HC_LIM_SUPERBEE = 5, HC_LIM_MC = 6,
  HC_LIM_VANLEER = 7,     /* harmonic-mean van Leer slope */
  HC_LIM_VANLEER_REF = 8, /* Limiters::VanLeer2 as written, limiters/limiter.ipp:81-89 */
  HC_LIM_CADA3 = 9
} hc_limiter;

/* Basis of the solution field: the SolVarT of SolutionField<SolVarT,2>
 * (solutionField/solutionField.h:56-91).  Gradients, reconstruction and limiting act on
 * the basis variables; fluxes reach the State through set2State of the basis
 * (conservationLaws/euler/transforms/primitive.ipp:24-60, conservationLaws/euler/transforms/conserved.ipp:31-76); the RK
 * update goes through the conserved set (spatial/eulerForwardUpdate.h:38-92).  State
 * uploads/downloads and ghost reference layers are in the basis.  Euler law only. */
typedef enum {
  HC_BASIS_PRIMITIVE = 0, /* {u, v, rho, p}, the reference drivers' choice (cylinder2D.cpp:110) */
  HC_BASIS_CONSERVED = 1  /* {rho u, rho v, rho, rho E} */
} hc_basis;

/* Runge-Kutta table (ODE::Explicit, ode.h:107-197) */
typedef enum { HC_RK_SSP11 = 0, HC_RK_SSP22 = 1, HC_RK_SSP33 = 2, HC_RK_SSP34 = 3 } hc_rk;

/* HC_FP64_DF: FP64 state, residuals and update (the FP64 interface); gradients,
 * reconstruction and fluxes in double-float (pairs of FP32, ~2^-47 relative
 * rounding, FP32 exponent range) on the FP32 pipes.  Single-mesh contexts only;
 * the stage kernel uses the 8x32 tile whatever the tile setting. */
typedef enum { HC_FP64 = 0, HC_FP32 = 1, HC_FP64_DF = 2 } hc_precision;

/* global: dt = cfl / max(lambda/V) at stage 0 (timestepping/rungeKutta.h:131-133);
 * local: per-cell cfl/lambda (spatial/eulerForwardUpdate.h:117-168) */
typedef enum { HC_DT_GLOBAL = 0, HC_DT_LOCAL = 1 } hc_dtmode;

/* Boundary condition of a mesh side (EulerBCs, conservationLaws/euler/euler.h:31-41).
 * Sides: 0 = i low, 1 = i high, 2 = j low, 3 = j high; periodic pairs (0,1), (2,3). */
typedef enum { HC_BC_PERIODIC = 0, HC_BC_FIXED = 1, HC_BC_RIEMANN = 2, HC_BC_ENTROPY = 3, HC_BC_WALL = 4 } hc_bc;

/* Conservation law (LawType).  HC_LAW_SCALAR is ScalarAdvection
 * (conservationLaws/scalarAdvection/scalarAdvection.h:45-98): an advected scalar q
 * with its advecting velocity, constant in time; its states are 3 planes of the
 * conserved set {u, v, q} (reference layers 3 planes per side, hc_residual 4
 * planes: 3 flux sums and lambda); fluxes HC_FLUX_RUSANOV or HC_FLUX_CENTRAL;
 * boundaries periodic, fixed or Riemann (inflow takes the reference value,
 * outflow the interior one, scalarAdvection/boundary/riemann.ipp); HC_FP64 or
 * HC_FP32; single-mesh contexts, no adjoint. */
typedef enum { HC_LAW_EULER = 0, HC_LAW_SCALAR = 1 } hc_law;

typedef struct {
  int flux;      /* hc_flux */
  int limiter;   /* hc_limiter */
  int rk;        /* hc_rk */
  int precision; /* hc_precision */
  int dt_mode;   /* hc_dtmode */
  double cfl;    /* UnsteadyTimeControls::cfl (controls.h:11-19) */
  int law;       /* hc_law; 0 = Euler */
  int basis;     /* hc_basis of the state and ghost layers; 0 = primitive */
} hc_config;

typedef struct {
  double dt;        /* last global dt (global mode) or the smallest local dt */
  double t;         /* accumulated time (global mode) */
  double resnorm;   /* L2 norm of the stage-0 density residual of the last step */
  int status;       /* hc_status of the device checks */
  int bad_cell;     /* first non-physical cell when status == HC_ERR_NONPHYSICAL */
  long long kernel_launches; /* kernels this context has launched so far */
} hc_step_stats;

/* Context lifetime.  Replaces the integrate() set-up of timestepping/rungeKutta.h:37-95. */
int hc_context_create(const hc_config* cfg, hc_ctx** out);
int hc_context_destroy(hc_ctx* ctx);
/* Run the context's kernels on this CUDA stream (a cudaStream_t; NULL = the legacy
 * default stream).  A new context runs on a non-blocking stream of its own, which
 * hc_get_stream returns. */
int hc_set_stream(hc_ctx* ctx, void* stream);
int hc_get_stream(hc_ctx* ctx, void** stream);

/* Mesh<2,Real> nodes (mesh/mesh.h:19-57); cells and face metrics are derived on the
 * device: geom::volume/surface, dual, xmetrics (geometry/volume.ipp:25-66,
 * geometry/surface.ipp:12-29, mesh/dual.ipp:42-83, spatial/lsqMetrics.h:31-163). */
int hc_mesh_upload(hc_ctx* ctx, int ni, int nj, const double* nodes_xy);

/* Mesh<1,Real> nodes (mesh/generate/oneD.h:11-36): the one-dimensional Euler path
 * (interiorResidual, spatial/residualCalc.h:74-127, with the 1D boundary loops and LSQ
 * metrics).  nc cells between increasing nodes x[0..nc]; the state is 3 planes {u, rho, p}
 * (the nDim = 1 primitive set), the residual 3 flux planes {rho u, rho, rho E} and the
 * spectral-radius sum; hc_set_bcs reads sides 0 (left) and 1 (right) only, ref[s] holding 3
 * values.  Euler law, FP64 or FP32, primitive basis; every flux, limiter, RK table, dt mode
 * and boundary type of the 2D path (no adjoint, dual time or branch signatures). */
int hc_mesh_upload_1d(hc_ctx* ctx, int nc, const double* nodes_x);

/* Species<Euler> (conservationLaws/euler/euler.h:48-60): gamma, R, minf. */
int hc_set_species(hc_ctx* ctx, double gamma, double gas_constant, double minf);

/* The AusmPlusUP<VFluxScaling, PFluxScaling> template arguments (hc_scaling) and the
 * Species<Euler> fields lref and dt that its adaptive scaling reads, mu = lref/(as dt)
 * (conservationLaws/euler/fluxes/ausmPlusUP.ipp:61-87).  Defaults: Convective,
 * Convective, lref 1, dt the largest double (conservationLaws/euler/species.ipp:12). */
int hc_set_low_mach(hc_ctx* ctx, int velocity_scaling, int pressure_scaling, double lref, double dt);

/* SolutionField::bcTypes and the reference layer of SolutionField::boundary
 * (solutionField/solutionField.h:56-91).  ref[side] holds 4 planes of values in the
 * context's basis (hc_config.basis), one per boundary face (nj faces on sides 0/1, ni
 * on 2/3); NULL for periodic or wall sides. */
int hc_set_bcs(hc_ctx* ctx, const int bc_type[4], const double* const ref[4]);

/* SolutionField::interior, 4 planes in the context's basis: primitive {u, v, rho, p}
 * (HC_BASIS_PRIMITIVE, the default) or conserved {rho u, rho v, rho, rho E}. */
int hc_state_upload(hc_ctx* ctx, const double* prim_soa);
int hc_state_download(hc_ctx* ctx, double* prim_soa);
/* Same through device pointers of the context's precision (no host copy). */
int hc_state_upload_device(hc_ctx* ctx, const void* prim_soa_device);
int hc_state_download_device(hc_ctx* ctx, void* prim_soa_device);

/* One residual evaluation of the current state: residualCalc (spatial/residualCalc.h:27-69)
 * including the boundary update (spatial/boundary/boundaryUpdate.h:137-266).
 * out: 5 planes -- 4 conserved flux sums and the spectral-radius sum. */
int hc_residual(hc_ctx* ctx, double* out5);

/* nsteps explicit RK steps: the time loop of integrate() (timestepping/rungeKutta.h:96-164). */
int hc_step(hc_ctx* ctx, int nsteps, hc_step_stats* stats);
/* The accumulated time t that hc_step_stats reports (the time integrate() accumulates,
 * timestepping/rungeKutta.h:96-164); uploading a mesh sets it to 0.  A run restored from
 * a checkpoint sets it to resume. */
int hc_set_time(hc_ctx* ctx, double t);
/* Enqueue nsteps without waiting; hc_sync waits and reports. */
int hc_step_async(hc_ctx* ctx, int nsteps);
/* nsteps RK steps of a host-resident field, the way integrate() advances the caller's
 * SolutionField in place (timestepping/rungeKutta.h:37-51): state_in (the solution basis's
 * planes, as hc_state_upload takes them) is copied to the device, stepped, and the result
 * copied to state_out (which may be state_in), with one synchronisation at the end; page-
 * locked host buffers let both copies run asynchronously.  stats as hc_step reports them. */
int hc_step_host(hc_ctx* ctx, int nsteps, const double* state_in, double* state_out, hc_step_stats* stats);
int hc_sync(hc_ctx* ctx, hc_step_stats* stats);

/* SteadyTimeControls (controls.h:31-48), which the reference declares but no driver
 * consumes: RK steps in the context's timestep mode (normally HC_DT_LOCAL) until the
 * L2 norm of the stage-0 density residual falls to residual_drop times its value at
 * the first step, or max_steps steps.  The norm is read on the host every
 * check_every steps; history (may be NULL) receives those reads, at most
 * history_len of them.  use_residual_smoothing (1D contexts, FP64 or FP32): every RK
 * stage's residual is smoothed by hc_smooth_1d's implicit smoothing with alpha =
 * smoothing_factor (>= 1; ends periodic on a periodic line, one-neighbour otherwise)
 * before the stage update; the monitored norm is the unsmoothed stage-0 residual's. */
typedef struct {
  long long max_steps;        /* nTimesteps */
  double residual_drop;       /* residual_drop */
  int check_every;
  int use_residual_smoothing; /* use_residual_smoothing */
  double smoothing_factor;    /* smoothing_factor: the smoothing's alpha */
} hc_steady_controls;

typedef struct {
  double res0;          /* density-residual norm of the first step */
  double res;           /* at the last read */
  long long steps;      /* steps taken */
  long long history_len;/* entries written to history */
  int converged;        /* res <= residual_drop * res0 */
} hc_steady_stats;

int hc_steady_run(hc_ctx* ctx, const hc_steady_controls* controls, double* history, long long history_len,
                  hc_steady_stats* stats);

/* Residual smoothing of the reference's legacy 1D path (OLD.fieldOperations/
 * centralImplicitSmoothing.ipp:2-60, centralExplicitSmoothing.ipp:5-39) on device
 * memory: nplanes planes of n >= 2 values (plane stride n).  r1 may equal or overlap r0:
 * the explicit kind then smooths a copy of r0 taken from the stream-ordered allocator.
 * HC_SMOOTH_IMPLICIT: four weighted-Jacobi sweeps (omega 2/3) of
 * (1 - beta delta^2) r1 = r0, beta = (alpha^2 - 1)/4, the result times alpha;
 * HC_SMOOTH_EXPLICIT: r1 = r0 + gamma delta^2 r0, gamma = ((1 + 4 beta)/alpha - 1)/4.
 * ends: 'p' periodic line, 'a' ends normalised by their one neighbour, anything else
 * unscaled (the reference's GridControls1D::boundaryCondition).  Asynchronous on the
 * context's stream; the implicit sweeps take scratch from the stream-ordered allocator. */
typedef enum { HC_SMOOTH_IMPLICIT = 0, HC_SMOOTH_EXPLICIT = 1 } hc_smooth_kind;
int hc_smooth_1d(hc_ctx* ctx, int kind, const double* r0_device, double* r1_device, long long n, int nplanes,
                 double alpha, int ends);

/* spectralRadius (spatial/spectralRadius.h:19-48): out_device[0] = max over the
 * ncell cells of lambda_sum[c] / vol[c], the fold starting at the smallest
 * positive double.  All three pointers are device memory; the call is
 * asynchronous on `stream` (a cudaStream_t, NULL = legacy default stream) and
 * takes its reduction scratch from the stream-ordered allocator. */
int hc_spectral_radius(const double* lambda_sum_device, const double* vol_device, long long ncell,
                       double* out_device, void* stream);

/* hc_spectral_radius for callers that cannot allocate device memory -- code that
 * runs while a framework owns the whole device memory pool, a fixed-budget or
 * real-time loop that must not call cudaMalloc/cudaFree, or a stream being
 * captured where allocation is not allowed.  No counterpart in the reference.
 * It allocates nothing: its 32 KiB of reduction scratch is a static device array
 * that every GPU loading this library keeps until the process exits, which caps
 * ncell at 8,388,608 (larger sizes return HC_ERR_ARG).  The first call on a
 * device looks the array's device address up, so make that first call before
 * any stream capture.  The looked-up address is kept for the life of the process:
 * after cudaDeviceReset on a device, do not call this entry point on that device
 * again.  All calls share the array: calls that overlap on the GPU (other streams,
 * other threads) race. */
int hc_spectral_radius_noalloc(const double* lambda_sum_device, const double* vol_device, long long ncell,
                               double* out_device, void* stream);

/* Dual-time stepping: ODE::Implicit::MultiStep in physical time (ode.h:12-82) with explicit
 * pseudo-time iterations, the scheme of the reference's legacy 1D driver
 * (timestepping/dualTime.ipp:4-105, OLD.fieldOperations/dualTimeResidual.ipp:2-41) on this
 * path.  Each physical step solves b_0 Q(u)/dt - g_0 R(u) = -(b_1 Q_n + b_2 Q_{n-1})/dt +
 * g_1 R(u_n) (Q the conserved set, R the flux residual, times the cell volume) by RK steps of
 * the context's table in pseudo time, the context's cfl and dt mode, each pseudo step
 * dtau / (1 + b_0 dtau / dt) (dualTime.ipp:65-66; local pseudo steps take the physical term
 * into the spectral radius); the inner loop stops after inner_max steps or once the density
 * dual-time residual fell by inner_drop (checked every check_every steps; 0 = never).  The
 * first step of BDF2 takes u_{n-1} = u_n, as the reference's initialisation does. */
typedef enum { HC_BDF1 = 0, HC_BDF2 = 1, HC_TRAPEZIUM = 2 } hc_multistep;
typedef struct {
  int outer_steps;   /* physical steps */
  double dt;         /* physical timestep; <= 0: cfl_outer / max(lambda/V) of the initial state */
  double cfl_outer;
  int scheme;        /* hc_multistep: backwardDifference1/2, trapeziumRule2 (ode.h:34-82) */
  int inner_max;     /* pseudo-time steps per physical step at most */
  double inner_drop; /* stop once ||R*_rho|| <= inner_drop * its first value (0: run inner_max) */
  int check_every;   /* pseudo-time steps between convergence checks */
} hc_dual_time_controls;
typedef struct {
  long long outer_steps, inner_steps;
  int last_inner;          /* pseudo steps of the last physical step */
  double dt, t;            /* physical timestep and time advanced */
  double res0_last, res_last; /* first and last dual-time density residual norm of the last step */
} hc_dual_time_stats;
int hc_dual_time_run(hc_ctx* ctx, const hc_dual_time_controls* ctl, hc_dual_time_stats* stats);

/* Branch signatures for the parity report (no counterpart in the reference): one
 * residual evaluation of the current state through a recording instantiation of the
 * stage kernel (the stepping kernels are not changed by it) that writes, per face, which
 * branches its evaluation took: bits 0-15 the limiter pieces of the left side's four
 * variables (4 bits each: bit 3 = (a > 0), bits 0-2 the interval of b/a that selects the
 * limiter's expression), 16-31 the right side's, 32-35 the flux's branches (Roe:
 * Harten's fix on the u-a / u+a waves; SLAU: |M_L| > 1, |M_R| > 1, mean-speed Mach > 1;
 * AUSM+up: |M_L| > 1, |M_R| > 1, left critical speed below the right; others: right
 * spectral radius larger), 36-37 the far-field path of a ghost face (1 interior copy,
 * 2 supersonic upwind copy, 3 subsonic), bit 63 set for every face.  sig_i holds
 * (ni+1)*nj i-faces, sig_j ni*(nj+1) j-faces (host arrays).  Comparing them with the
 * oracle's (or another precision's) counts the faces and cells where a branch flipped.
 * arg_i / arg_j (both or neither may be NULL): the (a, b) arguments of each face's eight
 * limiter calls (left side's four variables, then the right side's), 16 doubles per
 * face, so that a flip can be told apart from round-off noise at a breakpoint.  Euler
 * law; allocates and frees device buffers per call. */
int hc_face_signatures(hc_ctx* ctx, unsigned long long* sig_i, unsigned long long* sig_j, double* arg_i,
                       double* arg_j);

/* Mesh generators: make_cylinder_mesh (mesh/generate/twoD.h:139-179), radial
 * spacing stretched geometrically when stretch != 1; make_linspace_mesh
 * (mesh/generate/twoD.h:15-40). */
int hc_mesh_cylinder_nodes(int nr, int nth, double rc, double rb, double stretch, double* nodes_xy);
int hc_mesh_linspace_nodes(int nx, int ny, double lox, double hix, double loy, double hiy, double* nodes_xy);

/* ---------------------------------------------------------------------------
 * Discrete adjoint.  No counterpart in the reference.  The objective J is
 * evaluated on nsteps RK steps from the context's current state (which is left
 * unchanged); its gradient with respect to that initial state and to the
 * fixed-ghost reference states comes from the hand-written reverse of the
 * residual and of the RK update, with the timestep of every step frozen at the
 * value of the forward run ("rates": the per-step max lambda/V, returned so a
 * finite-difference check can replay them).  Binomial checkpointing keeps
 * `snapshots` states.  HC_FP64 contexts, HC_FP64_DF contexts (forward, replayed
 * and recomputed steps in double-float stage arithmetic, the face reverse in
 * double-float, the other reverse passes in FP64) or HC_FP32 contexts (FP32
 * throughout; rates, timesteps and J in FP64).  Euler law: Roe or Rusanov
 * reversed by hand, SLAU, SLAU as written, AUSM+up and RoeUnprecWS by forward-mode
 * tangents of the flux (HC_FP64 and HC_FP32); periodic, fixed and wall boundaries,
 * and Riemann / entropy far fields (their ghost update reversed by tangents; HC_FP64
 * and HC_FP32).
 * Scalar advection: Rusanov or central, periodic / fixed / Riemann boundaries, L2 objective.
 * NoLimit1/2/3, van Albada, MinMod, van Leer; global timestep.
 * ------------------------------------------------------------------------- */
typedef enum { HC_OBJ_DRAG = 0, HC_OBJ_L2 = 1 } hc_objective_kind;

typedef struct {
  int kind;              /* hc_objective_kind */
  double scale;          /* drag: J = scale/N * sum_{n=1..N} wall force of q_n along dir */
  double dir[2];         /* drag: force direction */
  const double* target;  /* L2: J = sum_cells sum_v weight[v] (q_N - target)^2, target 4 planes (host;
                            3 for the scalar law) */
  double weight[4];
  int target_on_device;  /* L2: target (and a batch's targets[k]) is FP64 device memory, not host */
} hc_objective;

typedef struct {
  double J;
  long long forward_steps;   /* RK steps run forward, checkpointing recomputation included */
  long long adjoint_steps;
  long long kernel_launches;
  double ms_forward;         /* first forward sweep */
  double ms_total;           /* forward sweep + reverse sweep */
  double ms_recompute;       /* part of the reverse sweep spent re-advancing from checkpoints */
  long long replays;         /* reversed steps whose stage states were recomputed (no stage tape) */
  long long stage_tapes;     /* stage tapes allocated (hc_set_adjoint_tapes) */
  double ms_reverse;         /* the reverse sweep alone, from the reverse call's first work */
} hc_adjoint_stats;

/* The pressure force on the inviscid-wall sides of the current state along dir (the
 * momentum flux the wall faces' boundary flux carries, inviscidWall.ipp:33-72, summed over
 * every wall face); the drag coefficient is that along the freestream divided by
 * (rho U^2 / 2) times the body's length scale.  2D Euler contexts, primitive basis. */
int hc_wall_force(hc_ctx* ctx, const double dir[2], double* force);

/* J only; rates_in NULL = compute the timesteps (rates_out receives them, nsteps values). */
int hc_objective_forward(hc_ctx* ctx, int nsteps, const hc_objective* obj, const double* rates_in,
                         double* rates_out, double* J);
/* J and its gradient: q0_bar (4 planes of the primitive state) and ref_bar (per side 0..3,
 * 4 planes of nface values, concatenated; zero where the side is periodic or a wall).
 * Scalar advection contexts (Rusanov or central flux, HC_OBJ_L2 on the conserved set
 * {u, v, q} with weight[0..2]; periodic, fixed or Riemann sides): 3 planes each. */
int hc_adjoint_gradient(hc_ctx* ctx, int nsteps, int snapshots, const hc_objective* obj, const double* rates_in,
                        double* q0_bar, double* ref_bar, double* rates_out, hc_adjoint_stats* stats);
/* hc_adjoint_gradient in two calls: record runs the forward sweep (J, rates_out) and keeps
 * its checkpoints in the context; reverse runs the reverse sweep from them without repeating
 * the forward sweep, writes q0_bar and ref_bar (layouts as above; NULL to skip) to host
 * memory or, with on_device, to FP64 device memory (asynchronous on the context's stream),
 * and releases the recording.  A new record, a mesh upload or destroy drops an unreversed
 * recording. */
int hc_adjoint_record(hc_ctx* ctx, int nsteps, int snapshots, const hc_objective* obj, const double* rates_in,
                      double* rates_out, double* J);
/* Stage tapes of the adjoint's checkpointing.  Reversing a step needs its stage states;
 * without a tape they are recomputed from the step's start state (a replay of all stages
 * but the last).  A stage tape keeps them (the start state and nst-1 stage states) from the
 * forward sweep or the re-advance that computed the step last before its reversal: the
 * last step of every re-advance and of the sweep's part before each stored checkpoint.
 * -1 (default): snapshots + 1 tapes, enough that no step is replayed, as many of them as fit
 * in half the free device memory at record time; 0: none (every step replayed, `snapshots`
 * states the only storage); k: at most k live at once.  Each tape holds nst states of the
 * mesh, allocated at record time.  Not in the reference (no adjoint). */
int hc_set_adjoint_tapes(hc_ctx* ctx, int ntapes);

/* The FP32 stage's tile loads staged by TMA tensor copies (on, the default, where the mesh's
 * rows are a multiple of 16 bytes) or plain per-thread loads (0): the same results bit for
 * bit, for comparison.  No counterpart in the reference. */
int hc_set_staged_loads(hc_ctx* ctx, int on);

/* Test hook of the failure detection (no counterpart in the reference): with on != 0 the
 * FP32 stage kernel whose loads are staged by TMA tensor copies (8x32 tiles, the common
 * limiters, nj a multiple of 4) arms its face-record barrier for 16 bytes more than the copy
 * delivers.  Every CTA's bounded wait (one second) then runs out, the step's status becomes
 * HC_ERR_TIMEOUT and hc_step returns it; no copy is left in flight and the context stays
 * usable.  0 (the default) clears it. */
int hc_inject_stalled_copy(hc_ctx* ctx, int on);
int hc_adjoint_reverse(hc_ctx* ctx, double* q0_bar, double* ref_bar, int on_device, hc_adjoint_stats* stats);

/* ---------------------------------------------------------------------------
 * Batched path: many independent meshes of uneven sizes in one set of buffers.
 * No counterpart in the reference (it runs one mesh per process).  Each instance
 * has its own mesh, boundary conditions, state and global dt; all instances
 * share the configuration and the species.  One persistent launch per RK stage
 * walks the tiles of every instance; a step sequence can be captured in a CUDA
 * graph and replayed.  HC_BATCH_PER_INSTANCE runs the same kernels as plain
 * per-instance launches, for comparison.
 * ------------------------------------------------------------------------- */
typedef struct hc_batch hc_batch;

typedef enum { HC_BATCH_PERSISTENT = 0, HC_BATCH_PER_INSTANCE = 1 } hc_batch_mode;
typedef enum { HC_ORDER_NATURAL = 0, HC_ORDER_LARGEST_FIRST = 1 } hc_batch_order;
/* HC_TILE_16x16_H: 16 x 16 cells run by 128 threads (single-mesh contexts only) */
typedef enum { HC_TILE_8x32 = 0, HC_TILE_4x32 = 1, HC_TILE_16x16 = 2, HC_TILE_16x16_H = 3 } hc_tile;

typedef struct {
  int tile;         /* hc_tile: cells per CTA tile */
  int ctas_per_sm;  /* persistent grid = SM count x ctas_per_sm */
  int order;        /* hc_batch_order of the work list */
  float ms_per_step;/* measured by hc_batch_autotune (0 when not measured) */
} hc_schedule;

/* Tile shape (hc_tile) of a single-mesh context's stage kernels: the FP64 and FP32
 * 2D stage, residual and adjoint-recompute launches (the double-float and 1D kernels
 * keep their own).  Defaults: HC_TILE_16x16_H in FP64 (16 x 16 cells, whose 544 faces
 * fill whole warps, on 128 threads: four CTAs per SM), HC_TILE_8x32 in FP32.  Every shape
 * gives the same results. */
int hc_set_tile(hc_ctx* ctx, int tile);

/* Corrections of two defects of the reference, off by default so that the reference's
 * results are reproduced as it computes them.  Not in the reference.
 * HC_FIX_MACH_SPLIT_P1: MachSplit_P1 (conservationLaws/euler/fluxes/machSplittings.ipp:26-31)
 *   is (M1 + eps)/(|M| + eps) with eps = numeric_limits<Real>::max(), which rounds to 1 for
 *   both signs: on supersonic faces SLAU and AUSM+up add the pressure of both sides, so
 *   F(q, q) differs from the exact flux by p n.  Corrected, P1 is M1/M, 1 upwind and 0
 *   downwind: (s M1 + eps)/(|M| + eps) with eps the smallest normal value.
 * HC_FIX_FARFIELD_TRANSVERSE: the Riemann and entropy far fields
 *   (conservationLaws/euler/boundary/riemann.ipp:48-50, entropy.ipp:47-49) copy the interior
 *   state when u_n/|u| is below a threshold, without the absolute value, so every outflow
 *   face copies the interior and a subsonic outflow receives nothing from the far field.
 *   Corrected, the test is |u_n|/|u| and outflow faces get the characteristic update.
 * The face-frame Roe dissipation is a flux of its own, HC_FLUX_ROE_FACE.  Applies from the
 * next step; batches take the same mask through hc_batch_set_corrections. */
typedef enum { HC_FIX_MACH_SPLIT_P1 = 1, HC_FIX_FARFIELD_TRANSVERSE = 2, HC_FIX_ALL = 3 } hc_fix;
int hc_set_corrections(hc_ctx* ctx, unsigned mask);

/* ninst meshes; nodes[k] as for hc_mesh_upload; bc[4k..4k+3] and ref[4k..4k+3]
 * as for hc_set_bcs (ref entries may be NULL where hc_set_bcs allows it).  cfg->law
 * HC_LAW_SCALAR: scalar advection instances (Rusanov or central flux; periodic, fixed
 * or Riemann sides; states and reference layers of 3 planes {u, v, q}). */
int hc_batch_create(const hc_config* cfg, int ninst, const int* ni, const int* nj, const double* const* nodes,
                    const int* bc, const double* const* ref, double gamma, double gas_constant, double minf,
                    hc_batch** out);
int hc_batch_destroy(hc_batch* b);
int hc_batch_set_stream(hc_batch* b, void* stream);
int hc_batch_state_upload(hc_batch* b, int inst, const double* prim_soa);
int hc_batch_state_download(hc_batch* b, int inst, double* prim_soa);
int hc_batch_set_schedule(hc_batch* b, const hc_schedule* s);
int hc_batch_set_corrections(hc_batch* b, unsigned mask);  /* hc_set_corrections for a batch */
int hc_batch_get_schedule(hc_batch* b, hc_schedule* s);
/* Enqueue nsteps RK steps of every instance (hc_batch_mode). */
int hc_batch_step_async(hc_batch* b, int nsteps, int mode);
/* Capture nsteps persistent steps into a CUDA graph (replacing any earlier one) and replay it. */
int hc_batch_graph_capture(hc_batch* b, int nsteps);
int hc_batch_graph_launch(hc_batch* b);
/* Wait; stats may be NULL or hold ninst entries (per-instance dt, t, status). */
int hc_batch_sync(hc_batch* b, hc_step_stats* stats);
/* Time every schedule candidate on `steps` persistent steps from the current
 * states (restored afterwards), keep the fastest and return it. */
int hc_batch_autotune(hc_batch* b, int steps, hc_schedule* best);
long long hc_batch_kernel_launches(hc_batch* b);

/* Discrete adjoint of every instance of a batch at once (no counterpart in the
 * reference): the objective of each instance is the L2 distance of its state after
 * nsteps RK steps to its own target (obj->kind HC_OBJ_L2, obj->weight; targets[k]
 * 4 planes of instance k, host), each instance with its own frozen global dt.  The
 * instances share the checkpoint schedule (`snapshots` states of the whole batch),
 * forward steps are the batch's persistent stage launches and every reverse pass is
 * one launch over all instances.  J[k] and q0_bar[k] (4 planes of the primitive
 * state; NULL entries skipped) per instance; stats: summed J, launches and times.
 * Supported as for hc_adjoint_gradient (HC_FP64 or HC_FP32 batches).  The batch's
 * states are left unchanged. */
int hc_batch_adjoint_gradient(hc_batch* b, int nsteps, int snapshots, const hc_objective* obj,
                              const double* const* targets, double* J, double* const* q0_bar,
                              hc_adjoint_stats* stats);
/* hc_batch_adjoint_gradient in two calls, for a differentiable forward whose backward comes
 * later (torch.autograd.Function): record runs the forward sweep (J[k] to the host) and keeps
 * its checkpoints in the batch; reverse runs the reverse sweep from them, writing q0_bar[k]
 * to host memory or, with on_device, to FP64 device memory (asynchronous on the batch's
 * stream), and releases them.  The forward sweep is not repeated.  A new record, or destroy,
 * drops an unreversed recording. */
int hc_batch_adjoint_record(hc_batch* b, int nsteps, int snapshots, const hc_objective* obj,
                            const double* const* targets, double* J);
int hc_batch_adjoint_reverse(hc_batch* b, double* const* q0_bar, int on_device, hc_adjoint_stats* stats);
int hc_batch_set_adjoint_tapes(hc_batch* b, int ntapes);  /* hc_set_adjoint_tapes for a batch */
/* instance k's state from FP64 device memory (asynchronous on the batch's stream) */
int hc_batch_state_upload_device(hc_batch* b, int inst, const double* prim_soa_device);

/* One interface flux evaluated on the host with the pointwise functions the stage kernels
 * compile: FluxInterface::flux(species, face, ql, qr) (conservationLaws/base/base.h:370-397)
 * of the flux `flux` (hc_flux) as the reference writes it (no corrections), for the C++
 * adapter's flux tags and for checks.  vscale, pscale: AUSM+up's LowMachScaling pair;
 * species {gamma, R, minf, lref, dt}; face {area, centre x, centre y, normal x, normal y,
 * tangent x, tangent y}; ql, qr primitive {u, v, rho, p}; out5 = {4 conserved flux
 * components times the area, lambda times the area}. */
int hc_flux_eval(int flux, int vscale, int pscale, const double species[5], const double face[7], const double ql[4],
                 const double qr[4], double out5[5]);
/* One slope limiter on the host, Limiter::limit(a, b) (limiters/limiter.h:14-28,
 * limiters/limiter.ipp:8-161; HC_LIM_VANLEER the harmonic-mean slope). */
int hc_limit_eval(int limiter, double a, double b, double* out);

const char* hc_last_error_string(void);
const char* hc_version(void);

#ifdef __cplusplus
}
#endif
#endif /* HC_H */
