/*
 * gbo.h -- C ABI of the GB300-native NonhydrostaticModel time-stepping library
 * (libgb300ocean.so).
 *
 * The library replaces the device side of Oceananigans.jl's
 * `time_step!(model::NonhydrostaticModel{<:RungeKutta3TimeStepper}, Δt)`
 * for RectilinearGrid / ImmersedBoundaryGrid(GridFittedBottom) models with
 * Periodic x and y and Bounded (or Flat) z.  A host binding (Julia `ccall`,
 * Python `ctypes`) keeps the reference's model API -- construction, `set!`,
 * `time_step!`, `run!` -- and calls only these entry points.
 *
 * Conventions
 *   - Plain C types only: pointers, sizes, enums.  No CUDA or torch types.
 *   - Every entry point returns GBO_OK (0) or a negative GBO_ERR_* code and
 *     never aborts; gbo_last_error() gives the message.  This mirrors the
 *     reference throwing ArgumentError at construction
 *     (src/Models/NonhydrostaticModels/nonhydrostatic_model.jl:150-175).
 *   - Arrays crossing the boundary hold interior points only, column-major
 *     with x fastest (Julia layout): index i + Nx*(j + Ny*k), 0-based.
 *     w carries Nz+1 vertical faces on Bounded z (Face location,
 *     src/Grids/grid_utils.jl:74-80); all other fields carry Nz levels.
 *   - A handle is not thread-safe; distinct handles may be driven from
 *     distinct host threads.  Work is issued on one CUDA stream per handle.
 */
#ifndef GBO_H
#define GBO_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define GBO_OK                 0
#define GBO_ERR_INVALID       -1  /* invalid argument or unsupported configuration */
#define GBO_ERR_CUDA          -2  /* a CUDA runtime call failed */
#define GBO_ERR_NAN           -3  /* NaN / Inf detected in the prognostic state */
#define GBO_ERR_NOT_CONVERGED -4  /* iterative pressure solver hit maxiter */
#define GBO_ERR_TIMEOUT       -5  /* a bounded device-side wait ran out */
#define GBO_ERR_NO_DEVICE     -6  /* no CUDA device visible */
#define GBO_ERR_STATE         -7  /* call out of order (e.g. stepping before set) */

/* ---- enums --------------------------------------------------------------- */
enum gbo_topology   { GBO_FLAT = 0, GBO_PERIODIC = 1, GBO_BOUNDED = 2 };
enum gbo_float_type { GBO_FLOAT32 = 4, GBO_FLOAT64 = 8 };
enum gbo_advection  { GBO_ADVECTION_NONE = 0, GBO_ADVECTION_CENTERED2 = 2, GBO_ADVECTION_WENO5 = 5 };
enum gbo_closure    { GBO_CLOSURE_NONE = 0, GBO_CLOSURE_SMAGORINSKY_LILLY = 1,
                      GBO_CLOSURE_AMD = 2, GBO_CLOSURE_SCALAR_DIFFUSIVITY = 3,
                      GBO_CLOSURE_DYNAMIC_SMAGORINSKY = 4 };
/* DynamicSmagorinsky averaging (dynamic_coefficient.jl:104-117): over x and y, or
 * along Lagrangian trajectories (the reference's default, not available on GB300) */
enum gbo_averaging  { GBO_AVERAGING_XY = 0, GBO_AVERAGING_LAGRANGIAN = 1 };
enum gbo_timestepper { GBO_TIMESTEPPER_RK3 = 0, GBO_TIMESTEPPER_QAB2 = 1 };
enum gbo_solver     { GBO_SOLVER_FFT = 0, GBO_SOLVER_FOURIER_TRIDIAGONAL = 1,
                      GBO_SOLVER_CONJUGATE_GRADIENT = 2 };
enum gbo_precond    { GBO_PRECOND_FFT = 0, GBO_PRECOND_NONE = 1, GBO_PRECOND_LEARNED = 2 };

/* field identifiers for set/get */
#define GBO_FIELD_U      0
#define GBO_FIELD_V      1
#define GBO_FIELD_W      2
#define GBO_FIELD_TRACER 3        /* tracer n is GBO_FIELD_TRACER + n */
#define GBO_FIELD_PNHS   100      /* nonhydrostatic pressure (model.pressures.pNHS) */
#define GBO_FIELD_PHY    101      /* hydrostatic pressure anomaly (model.pressures.pHY′) */
#define GBO_FIELD_NU     102      /* eddy viscosity νₑ (closure_fields.νₑ) */
#define GBO_FIELD_KAPPA  103      /* AMD tracer diffusivity κₑ of tracer 0 */
#define GBO_FIELD_JLM    104      /* 𝒥ᴸᴹ of a Lagrangian-averaged DynamicSmagorinsky (closure_fields.𝒥ᴸᴹ) */
#define GBO_FIELD_JMM    105      /* 𝒥ᴹᴹ of a Lagrangian-averaged DynamicSmagorinsky (closure_fields.𝒥ᴹᴹ) */

#define GBO_MAX_TRACERS 4
/* Upper bound on conjugate-gradient iterations per pressure solve (the reference's
 * default maxiter is the number of cells; the device loop also stops here and
 * reports GBO_ERR_NOT_CONVERGED, so a stagnating solve ends in bounded time). */
#define GBO_CG_MAX_ITERATIONS 20000

/* Grid: replaces RectilinearGrid(size, x, y, z, topology) and
 * ImmersedBoundaryGrid(grid, GridFittedBottom(h))
 * (src/Grids/rectilinear_grid.jl:266-305; src/ImmersedBoundaries/grid_fitted_bottom.jl:17). */
typedef struct gbo_grid_desc {
    int32_t size[3];          /* Nx, Ny, Nz (Nz = 1 with topology[2] == GBO_FLAT) */
    int32_t topology[3];      /* x, y must be GBO_PERIODIC; z GBO_BOUNDED or GBO_FLAT */
    double  x[2], y[2], z[2]; /* domain extents (z ignored when z_faces != NULL) */
    const double* z_faces;    /* NULL: regular z; else Nz+1 increasing face positions */
    const double* bottom_height; /* NULL: no immersed boundary; else Nx*Ny bottom heights h(x,y) */
    int32_t float_type;       /* GBO_FLOAT32 or GBO_FLOAT64 */
} gbo_grid_desc;

/* Model physics: replaces NonhydrostaticModel(grid; advection, closure, buoyancy,
 * coriolis, tracers, boundary_conditions, pressure_solver)
 * (src/Models/NonhydrostaticModels/nonhydrostatic_model.jl:124-313). */
typedef struct gbo_model_desc {
    int32_t advection;               /* gbo_advection: only GBO_ADVECTION_WENO5 is implemented (the
                                        default here; the reference's own default is Centered()) */
    int32_t closure;                 /* gbo_closure */
    double  closure_C;               /* Smagorinsky C (0.16) or AMD C (1/3) */
    double  closure_Cb;              /* Lilly reduction factor Cb (1.0); 0 gives the constant-coefficient
                                        Smagorinsky(coefficient = C); unused by AMD */
    double  closure_Pr;              /* turbulent Prandtl number for all tracers (1.0) */
    int32_t ntracers;                /* 0..GBO_MAX_TRACERS */
    int32_t buoyancy_tracer;         /* 1: tracer 0 is the BuoyancyTracer `b`; 0: no buoyancy */
    int32_t has_coriolis;            /* 1: FPlane(f) with the EnstrophyConserving scheme */
    double  coriolis_f;
    double  tracer_flux_top[GBO_MAX_TRACERS];    /* FluxBoundaryCondition values (top) */
    double  tracer_flux_bottom[GBO_MAX_TRACERS]; /* FluxBoundaryCondition values (bottom) */
    int32_t pressure_solver;         /* gbo_solver */
    int32_t preconditioner;          /* gbo_precond, CG only */
    double  cg_reltol;               /* 0 -> sqrt(eps(FT)) as the reference defaults */
    double  cg_abstol;               /* 0 -> sqrt(eps(FT)) */
    int32_t cg_maxiter;              /* 0 -> Nx*Ny*Nz */
    /* ScalarDiffusivity(ν, κ) with constant coefficients, isotropic and explicit
     * (turbulence_closure_implementations/scalar_diffusivity.jl:8-80) */
    double  closure_nu;
    double  closure_kappa[GBO_MAX_TRACERS];
    /* timestepper = :RungeKutta3 (default) or :QuasiAdamsBashforth2 with χ
     * (src/TimeSteppers/quasi_adams_bashforth_2.jl:39-48; default χ = 0.1) */
    int32_t timestepper;             /* gbo_timestepper */
    double  ab2_chi;
    /* DynamicSmagorinsky(averaging = (1, 2), schedule = IterationInterval(1)): the
     * coefficient is averaged over x and y per level and recomputed at every state
     * update; minimum_numerator bounds its numerator from below (1e-32)
     * (turbulence_closure_implementations/Smagorinskys/dynamic_coefficient.jl:1-20,
     * 215-275; scale_invariant_operators.jl).  Uses closure_Pr; ignores C and Cb. */
    double  closure_min_numerator;
    int32_t closure_averaging;       /* a gbo_averaging; LAGRANGIAN by default, as for DynamicSmagorinsky() */
} gbo_model_desc;

typedef struct gbo_model gbo_model;

/* Fill *d with the reference's defaults: WENO5, no closure, no tracers, FFT solver. */
void gbo_model_desc_default(gbo_model_desc* d);

/* The conjugate-gradient stopping parameters a model of this grid and descriptor uses,
 * with zeros replaced by the reference's defaults: reltol = abstol = sqrt(eps(FT)) and
 * maxiter = Nx*Ny*Nz (ConjugateGradientPoissonSolver(grid; reltol, abstol, maxiter),
 * src/Solvers/conjugate_gradient_poisson_solver.jl:134-137, conjugate_gradient_solver.jl:91;
 * the reference's summary shows them, conjugate_gradient_poisson_solver.jl:55-57).
 * Host only; no device is needed. */
int gbo_cg_parameters(const gbo_grid_desc* grid, const gbo_model_desc* desc, double* reltol, double* abstol,
                      double* maxiter);

/* Construct a model on the current CUDA device.
 * Replaces NonhydrostaticModel(grid; ...) (nonhydrostatic_model.jl:124). */
int gbo_model_create(const gbo_grid_desc* grid, const gbo_model_desc* desc, gbo_model** out);

/* Release all device memory held by the model. */
void gbo_model_destroy(gbo_model* m);

/* Copy interior values of one field from host memory (dtype GBO_FLOAT32/64).
 * Replaces set!(field, array) (src/Fields/set!.jl:46-70) for one field. */
int gbo_set_field(gbo_model* m, int32_t field, const void* host, int32_t dtype, int64_t count);

/* Finish `set!(model; kwargs...)`: mask immersed cells, update the state and,
 * if enforce_incompressibility, project the velocities onto the divergence-free
 * space (compute_pressure_correction!(model, 1) + make_pressure_correction!)
 * and update again (src/Models/NonhydrostaticModels/set_nonhydrostatic_model.jl:39-74). */
int gbo_set_finalize(gbo_model* m, int32_t enforce_incompressibility);

/* Copy interior values of one field to host memory (dtype GBO_FLOAT32/64). */
int gbo_get_field(gbo_model* m, int32_t field, void* host, int32_t dtype, int64_t count);

/* Number of interior values of `field` (for sizing host buffers). */
int64_t gbo_field_count(const gbo_model* m, int32_t field);

/* Device pointer and element count of a field (zero-copy access for a host binding's
 * unsafe_wrap / torch view).  The element type is the model's float type.
 * Tracers of GBO_FLOAT32 models on a Bounded z are stored as departures from a
 * per-level reference profile (the horizontal mean of the values the tracer was last
 * set to): the device array holds c - profile[k], and gbo_get_field returns the sum.
 * A stratification b = N² z + b′ held directly in FP32 would round b′ at the ulp of
 * N² z on every stage; as departures it is rounded at the ulp of b′. */
int gbo_field_device_pointer(gbo_model* m, int32_t field, void** dptr, int64_t* count);

/* The reference profile (Nz values, FP64) of a tracer field: zeros where the tracer
 * is stored as it is (GBO_FLOAT64 models, Flat z).  No counterpart in the reference,
 * which stores every tracer directly. */
int gbo_field_reference_profile(gbo_model* m, int32_t field, double* out, int64_t count);

/* Advance nsteps RK3 time steps of size dt.
 * Replaces time_step!(model::AbstractModel{<:RungeKutta3TimeStepper}, Δt)
 * (src/TimeSteppers/runge_kutta_3.jl:103-168) with the NonhydrostaticModel substep
 * (src/Models/NonhydrostaticModels/nonhydrostatic_rk3_substep.jl:31-63). */
int gbo_time_step(gbo_model* m, double dt, int32_t nsteps);

/* Clock (model.clock.time, model.clock.iteration; src/TimeSteppers/clock.jl). */
int gbo_clock(const gbo_model* m, double* time, int64_t* iteration);

/* Block until all work issued for the model has finished; returns the first
 * deferred device error (NaN flag, solver non-convergence, CUDA error). */
int gbo_synchronize(gbo_model* m);

/* Iterations taken by the last conjugate-gradient pressure solve (0 for direct solvers). */
int32_t gbo_last_solver_iterations(const gbo_model* m);

/* Message describing the last error on this handle (or a global message if m is NULL). */
const char* gbo_last_error(const gbo_model* m);

/* Library version string. */
const char* gbo_version(void);

/* ---- checkpoint / restart ------------------------------------------------------
 * Replaces prognostic_state(model) / restore_prognostic_state!(model, state)
 * (src/Models/NonhydrostaticModels/nonhydrostatic_model.jl:354-377), which the
 * Checkpointer and run!(sim; pickup=true) use.  The state is one host buffer of
 * gbo_state_bytes(m) bytes: a header (clock, sizes, float type) and the interior
 * values of u, v, w, the tracers and pNHS (the conjugate-gradient initial guess).
 * RK3 needs no tendency history across steps (ζ₁ = 0); the closure fields and the
 * hydrostatic pressure anomaly are recomputed on restore, so a restored model
 * continues exactly as the original.  gbo_set_state rejects a buffer written by a
 * model of another size, float type or tracer count. */
int64_t gbo_state_bytes(const gbo_model* m);
int gbo_get_state(gbo_model* m, void* buf, int64_t bytes);
int gbo_set_state(gbo_model* m, const void* buf, int64_t bytes);

/* ---- simulation loop ------------------------------------------------------
 * run!(Simulation(model; Δt, stop_time, stop_iteration, wall_time_limit,
 * align_time_step)) with the default NaNChecker and an optional TimeStepWizard
 * callback (src/Simulations/run.jl:165-262, simulation.jl:68-119,
 * time_step_wizard.jl:66-115).  The loop runs on the device: Δt alignment with
 * stop_time, the step, the clock, the stop criteria, the NaN check and the
 * wizard's CFL reductions are nodes of one CUDA graph whose conditional WHILE
 * node repeats them, so the host waits only once per iterations_per_launch
 * iterations (where wall_time_limit is checked).  As in the reference at least
 * one step is taken per call, and a model at iteration 0 first evaluates every
 * callback once (initialize!(sim), run.jl:319-347). */
enum gbo_stop_reason { GBO_STOP_NONE = 0, GBO_STOP_TIME = 1, GBO_STOP_ITERATION = 2, GBO_STOP_NAN = 3,
                       GBO_STOP_WALL_TIME = 4 };
typedef struct gbo_run_desc {
    double  dt;                    /* Simulation(model; Δt): the first time step */
    double  stop_time;             /* INFINITY: none */
    double  stop_iteration;        /* INFINITY: none (a Float64, as in the reference) */
    double  wall_time_limit;       /* seconds; INFINITY: none */
    int32_t align_time_step;       /* 1: align Δt with stop_time (default) */
    double  minimum_relative_step; /* must be 0 (the default): skipped steps are not supported */
    int32_t nan_check_interval;    /* NaNChecker on u every N iterations (default 100; 0: none) */
    int32_t nan_erroring;          /* 1: a NaN makes gbo_run return GBO_ERR_NAN */
    int32_t wizard_interval;       /* TimeStepWizard callback on IterationInterval(N); 0: none */
    double  cfl, diffusive_cfl;    /* TimeStepWizard(cfl = 0.2, diffusive_cfl = Inf, */
    double  max_change, min_change;/*   max_change = 1.1, min_change = 0.5, */
    double  max_dt, min_dt;        /*   max_Δt = Inf, min_Δt = 0) */
    int32_t iterations_per_launch; /* iterations per graph launch (default 100) */
} gbo_run_desc;
typedef struct gbo_run_result {
    double  dt;                    /* simulation.Δt at the end (the wizard's last value) */
    double  time;                  /* model.clock.time */
    int64_t iteration;             /* model.clock.iteration */
    int64_t steps;                 /* steps taken by this call */
    int32_t stop_reason;           /* gbo_stop_reason of the first criterion met */
    int32_t nan_detected;
} gbo_run_result;
void gbo_run_desc_default(gbo_run_desc* d);
int gbo_run(gbo_model* m, const gbo_run_desc* d, gbo_run_result* out);

/* cell_advection_timescale(model) (src/Advection/cell_advection_timescale.jl:15-36)
 * and cell_diffusion_timescale(model) of the closure
 * (src/TurbulenceClosures/turbulence_closure_diagnostics.jl:48-63; Inf without a
 * closure), reduced on the device from the current state. */
int gbo_cell_advection_timescale(gbo_model* m, double* out);
int gbo_cell_diffusion_timescale(gbo_model* m, double* out);

/* ---- device-buffer entry points ------------------------------------------------
 * gbo_poisson_solve_device, gbo_poisson_operator_device, gbo_precondition_device and the
 * trainer's gradients / step read device buffers on the library's own stream.  Each
 * first orders that stream after the work already issued to the legacy default stream
 * (cudaStreamLegacy, where PyTorch's default stream and plain CUDA calls run), and each
 * returns after its results are written.  A caller that writes the inputs on another
 * stream synchronises that stream first.
 *
 * ---- standalone Poisson solve ---------------------------------------------
 * Solve ∇²ϕ = rhs with the model's pressure solver on device buffers holding
 * Nx*Ny*Nz interior values of the model's float type.
 * Replaces solve!(ϕ, solver::FFTBasedPoissonSolver / FourierTridiagonalPoissonSolver, b)
 * (src/Solvers/fft_based_poisson_solver.jl:94-124;
 *  src/Solvers/fourier_tridiagonal_poisson_solver.jl:231-260)
 * and, for the CG solver, solve!(x, ::ConjugateGradientPoissonSolver, rhs)
 * (src/Solvers/conjugate_gradient_poisson_solver.jl; the rhs there is V·div). */
int gbo_poisson_solve_device(gbo_model* m, void* phi_device, const void* rhs_device);

/* ---- learned preconditioner correction ---------------------------------------
 * No counterpart in the reference (its CG preconditioners are FFT-based, diagonal or
 * none).  For a model with the ConjugateGradientPoissonSolver and its FFT
 * preconditioner, gbo_learned_preconditioner loads a 3-D U-Net (four levels, 16, 32,
 * 48, 64 channels, 3³ kernels; BF16 on the tensor cores, FP32 accumulation) whose
 * output corrects the FFT preconditioner: z = z_fft + s_z net(r/s_r, z_fft/s_z,
 * active), s_r = RMS(r), s_z = RMS(z_fft).  The CG becomes the flexible (Polak-Ribière)
 * variant.  `weights` holds
 * gbo_learned_weight_count() FP32 values, per layer [cout][cin][3][3][3] then bias, in
 * the order enc0 (3→16), enc1 (16→32), enc2 (32→48), enc3 (48→64), dec3 (64→48),
 * dec2 (48→32), dec1 (32→16), out (16→1); NULL restores the plain FFT preconditioner.
 * Nx, Ny and Nz must be divisible by 8. */
int64_t gbo_learned_weight_count(void);
int gbo_learned_preconditioner(gbo_model* m, const float* weights, int64_t count);
/* out = V∇²x, the CG operator with the conditional differences of the immersed grid
 * (conjugate_gradient_poisson_solver.jl:111-137); device buffers of the model's float type. */
int gbo_poisson_operator_device(gbo_model* m, const void* x_device, void* out_device);
/* z = M r with the model's CG preconditioner (including a loaded learned correction). */
int gbo_precondition_device(gbo_model* m, const void* r_device, void* z_device);

/* ---- training the learned correction on the GPU ----------------------------------
 * No counterpart in the reference.  A trainer holds the network for an Nx × Ny × Nz
 * grid (divisible by 8) with FP32 master weights (initial values from `weights`, the
 * layout of gbo_learned_preconditioner) and Adam moments, and trains it with the
 * library's own kernels: the forward and data-gradient convolutions on the
 * fifth-generation tensor cores (tcgen05, BF16 operands, FP32 accumulation in TMEM),
 * weight gradients on BF16 tensor-core MMAs with FP32 accumulation, pooling /
 * up-sampling / ReLU backward passes, the loss and Adam.  One sample is a residual r,
 * its FFT-preconditioned z_fft and the error e = A⁻¹ r (the exact correction is
 * e - z_fft), with the active-cell mask `active` (1 or 0): device arrays of Nx*Ny*Nz
 * FP32 values, x fastest.  The loss is Σ d² / Σ t_c² with t = (e - z_fft) / s_z,
 * d = (net - t)·active and t_c = t·active, each less its active-cell mean.
 *   gbo_learned_trainer_gradients: the loss and d(loss)/d(weights) (host, same layout)
 *     of one sample, without updating;
 *   gbo_learned_trainer_step: one Adam step (β1 = 0.9, β2 = 0.999, ε = 1e-8) on one sample;
 *   gbo_learned_trainer_weights: the current FP32 weights (host). */
typedef struct gbo_learned_trainer gbo_learned_trainer;
int gbo_learned_trainer_create(int32_t nx, int32_t ny, int32_t nz, const float* weights, int64_t count,
                               gbo_learned_trainer** out);
void gbo_learned_trainer_destroy(gbo_learned_trainer* t);
int gbo_learned_trainer_gradients(gbo_learned_trainer* t, const float* r_device, const float* z_device,
                                  const float* e_device, const float* active_device, double* loss, float* grad);
int gbo_learned_trainer_step(gbo_learned_trainer* t, const float* r_device, const float* z_device,
                             const float* e_device, const float* active_device, double lr, double* loss);
int gbo_learned_trainer_weights(gbo_learned_trainer* t, float* weights);
/* The cudaStream_t (as void*) the trainer's work is issued on. */
int gbo_learned_trainer_stream(gbo_learned_trainer* t, void** stream);

/* ---- ensembles ---------------------------------------------------------------
 * No counterpart in the reference, which advances models one at a time.  An
 * ensemble owns n independent models (each created as by gbo_model_create from
 * grids[i], descs[i]; sizes and physics may differ) and advances all of them with
 * one CUDA graph launch per step: every member's step is a parallel branch of the
 * graph, so small members share the GPU instead of running back to back.
 * Members are ordinary handles for gbo_set_field / gbo_set_finalize /
 * gbo_get_field / gbo_clock; they belong to the ensemble (never pass them to
 * gbo_model_destroy) and are stepped only through gbo_ensemble_time_step. */
typedef struct gbo_ensemble gbo_ensemble;
int gbo_ensemble_create(int32_t n, const gbo_grid_desc* grids, const gbo_model_desc* descs, gbo_ensemble** out);
void gbo_ensemble_destroy(gbo_ensemble* e);
int32_t gbo_ensemble_size(const gbo_ensemble* e);
gbo_model* gbo_ensemble_member(gbo_ensemble* e, int32_t i);
/* The cudaStream_t (as void*) on which the ensemble graph is launched (instrumentation). */
int gbo_ensemble_stream(gbo_ensemble* e, void** stream);
/* Advance every member by nsteps steps of dt; returns the first member error (NaN,
 * CG non-convergence) after all members finished, with gbo_last_error(NULL) naming it. */
int gbo_ensemble_time_step(gbo_ensemble* e, double dt, int32_t nsteps);

/* ---- allocation-free FFT Poisson solve --------------------------------------
 * No counterpart in the reference: Oceananigans allocates the FFT solver's work
 * arrays when FFTBasedPoissonSolver(grid) is built, and gbo_poisson_solve_device
 * uses the work arrays gbo_model_create allocated.  This entry point solves
 * ∇²ϕ = rhs on a regular RectilinearGrid (Periodic x, y; Bounded or Flat z;
 * z_faces and bottom_height NULL) with the FFT-based solver and allocates no
 * memory: its work space is one static device array of
 * GBO_STATIC_SCRATCH_BYTES (32 MiB) in the library, and ϕ itself is the real
 * work buffer.  It is for callers that cannot allocate device memory at solve
 * time: a host whose device memory belongs to another allocator (a CUDA.jl or
 * PyTorch caching pool that already holds the free memory, where a cudaMalloc
 * from the library would fail or fragment the pool), and a caller with work in
 * flight on other streams, where cudaMalloc / cudaFree could synchronize the
 * device and stall that work.
 *   - phi_device, rhs_device: Nx*Ny*Nz interior values of grid->float_type
 *     (x fastest); phi may equal rhs (in place).  rhs is not modified otherwise.
 *   - cuda_stream: the cudaStream_t (as void*) the work is issued on; NULL is the
 *     default stream.  The call returns once the work is enqueued.
 *   - Grids whose work space exceeds GBO_STATIC_SCRATCH_BYTES are rejected with
 *     GBO_ERR_INVALID and a message giving the bytes needed (FP32: about
 *     (Nx/2+1)*Ny*Nz*8 bytes, e.g. up to 256x256x64, or 2048x2048 on a Flat z;
 *     FP64: twice that, e.g. 128^3, or 2048x1024 on a Flat z).
 *   - Every call looks up the static array's address in the current CUDA context
 *     (a host-side lookup, so a context reset or another current context is safe);
 *     the first call in each context also raises the pass kernels' shared-memory
 *     limits.  Make that first call before any stream capture.
 *   - The scratch is one array per device shared by all callers: calls that
 *     overlap in time (other streams, other threads) race on it and must be
 *     serialized by the caller.  Nothing in it has to start at zero; every
 *     value a call reads was written earlier in the same call. */
#define GBO_STATIC_SCRATCH_BYTES (32u * 1024u * 1024u)
int gbo_poisson_solve_fft_static(const gbo_grid_desc* grid, void* phi_device, const void* rhs_device,
                                 void* cuda_stream);

/* ---- instrumentation -----------------------------------------------------
 * No reference counterpart: the reference measures with external profilers
 * (benchmarking/, nsys in CI).  These expose what a benchmark harness needs to
 * time the library on the stream it launches on. */

/* The cudaStream_t (as void*) on which all of the model's work is issued. */
int gbo_model_stream(gbo_model* m, void** stream);

/* Cumulative number of CUDA kernels launched for this model (graph replays count
 * every kernel they contain). */
int64_t gbo_kernel_launches(const gbo_model* m);

/* Run nsteps time steps launching kernels one by one with CUDA events around each
 * kernel group; writes the mean duration per launch (ms) of group g into ms[g] for
 * g < min(nmax, gbo_kernel_group_count()).  Advances the model like gbo_time_step. */
int gbo_kernel_timings(gbo_model* m, double dt, int32_t nsteps, double* ms, int32_t nmax);
int32_t gbo_kernel_group_count(void);
/* Launches of each kernel group in the last gbo_kernel_timings pass (all its steps). */
int gbo_kernel_timing_counts(const gbo_model* m, int64_t* n, int32_t nmax);
const char* gbo_kernel_group_name(int32_t g);

/* Launch shapes of the spectral Poisson passes and of the fused tendency kernel.  The
 * pass tiles set speed only (every column and line is transformed by the same arithmetic
 * whatever the tile); the levels per block of the fused kernel change where a block
 * starts its vertical march, which can change results by rounding.  A model starts from
 * the tuned shape of its size
 * class (a table measured on GB300 and compiled into the library; see
 * oceananigans_gb300/autotune.py) or, for sizes not in the table, from the default rule. */
typedef struct gbo_launch_shape {
    int32_t dct_columns; /* x columns per block of the z DCT pass: a power of two, 2..64 */
    int32_t x_lines;     /* (y, z) lines per block of the x real-FFT pass: 1..32 */
    int32_t y_columns;   /* kx columns per block of the y FFT pass: a power of two, 1..64 */
    int32_t levels;      /* levels each block of the fused tendency kernel marches: 1..Nz (1 on a Flat z) */
} gbo_launch_shape;
int gbo_get_launch_shape(const gbo_model* m, gbo_launch_shape* out);
/* Replaces the shape (invalid: GBO_ERR_INVALID, model unchanged); the model's captured
 * step graphs are rebuilt at the next step.  Not for ensemble members. */
int gbo_set_launch_shape(gbo_model* m, const gbo_launch_shape* shape);

#ifdef __cplusplus
}
#endif

#endif /* GBO_H */
