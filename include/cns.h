/*
 * cns.h -- C ABI of the GB300 (sm_103a) time-advance path for the 3D compressible
 * Navier-Stokes equations (conservative split-form RHS + Runge-Kutta stage update).
 *
 * This header is the drop-in boundary for the host-side call sequence of
 * CudaNavierStokes (src/main.h:23-42, src/cuda_main.cu:109-186,249-265):
 *
 *   reference                                      this ABI
 *   ---------------------------------------------  -------------------------------------
 *   compile-time macros  src/globals.h:5-95        cns_params (runtime), cns_default_params
 *   setDevice + setGPUParameters + initSolver      cns_create
 *       (src/cuda_utils.cu:49-179,415-519,816)
 *   initGrid / derivGrid (src/init.cpp:32-92,258)  cns_get_grid (grid built inside cns_create)
 *   calculateSponge (src/sponge.cu:83-240)         cns_set_sponge_profiles / cns_set_sponge
 *   copyField(0) / copyField(1)                    cns_copy_field
 *       (src/cuda_utils.cu:299-370)
 *   runSimulationLowStorage / runSimulation        cns_run
 *       (src/cuda_main.cu:109-186, :44-107)
 *   calcRHS (src/cuda_main.cu:15-42)               cns_calc_rhs   (test hook)
 *   calcTimeStepPressGrad (src/cuda_main.cu:249)   cns_get_scalars (dt, dpdz, time)
 *   clearSolver (src/cuda_utils.cu:521-595)        cns_destroy
 *
 * Conventions
 *   - All fields are FP64, x fastest: index(i,j,k) = i + j*mx + k*mx*my
 *     (src/globals.h:60-61). The stored state is rho, primitive u, v, w and rho*E,
 *     exactly as the reference's d_r, d_u, d_v, d_w, d_e (src/cuda_main.h:14-18).
 *   - Host arrays are caller-owned; the library copies in and out. Device state is
 *     owned by the handle.
 *   - Every call returns an int status (CNS_OK = 0). cns_last_error() gives a
 *     thread-local message for the last failure on the calling thread.
 *   - A handle is used from one host thread at a time. Work is issued on the
 *     handle's stream (cns_set_stream); calls that return host data synchronise it.
 *   - The product path has no CPU fallback: without a usable CUDA device every
 *     entry point that needs one returns CNS_ERR_CUDA.
 */
#ifndef CNS_GB300_H_
#define CNS_GB300_H_

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define CNS_API __attribute__((visibility("default")))
#else
#define CNS_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define CNS_OK             0
#define CNS_ERR_INVALID    1   /* bad parameter or argument                         */
#define CNS_ERR_CUDA       2   /* CUDA runtime error / no device                     */
#define CNS_ERR_OOM        3   /* device allocation failed or HBM budget exceeded    */
#define CNS_ERR_NONFINITE  4   /* non-finite or non-physical state detected          */
#define CNS_ERR_TIMEOUT    5   /* a bounded device wait gave up                      */
#define CNS_ERR_STATE      6   /* call made in the wrong order (e.g. run before init) */

/* time schemes */
#define CNS_RK3_LOWSTORAGE 0   /* Wray low-storage RK3 (src/cuda_main.cu:10-11,109-186) */
#define CNS_RK3_CLASSIC    1   /* classic 3-stage RK3  (src/cuda_main.cu:44-107,188-216) */
#define CNS_RK4_CLASSIC    2   /* classic 4-stage RK4: no counterpart in the reference   */

/* RHS arithmetic */
#define CNS_PREC_FP64      0   /* plain FP64 everywhere, as the reference                */
#define CNS_PREC_FP32_RHS  1   /* RHS in FP32; state, RK accumulation, T/p recovery and
                                  reductions in FP64                                     */
#define CNS_PREC_PAIR_RHS  2   /* RHS in FP32-pair ("double-float", ~48-bit) arithmetic;
                                  state, RK accumulation, T/p recovery and reductions
                                  in FP64 (single solvers; batches take modes 0 and 1)   */

/*
 * Runtime mirror of the reference's compile-time parameter surface
 * (src/globals.h:14-58, src/sponge.h:4-17, src/perturbation.h:14-22).
 * Axis convention is the reference's: x is the only non-periodic / stretched /
 * wall-normal direction, y is periodic, z is periodic or (boundary layer)
 * extrapolated; the channel body force acts on z momentum.
 */
typedef struct cns_params {
    int32_t mx, my, mz;          /* mx_tot, my_tot, mz_tot (globals.h:24-26)            */
    double  Lx, Ly, Lz;          /* domain lengths (globals.h:21-23)                     */
    int32_t stencil_size;        /* S: advective half-width, order 2S, 1..4 (globals.h:18) */
    int32_t stencil_visc;        /* V: viscous half-width, order 2V, 1..S (globals.h:19)   */
    double  Re, Pr, Ma, gam, viscexp;   /* globals.h:42-46                               */
    double  cfl;                 /* CFL (globals.h:29)                                   */
    int32_t scheme;              /* CNS_RK3_LOWSTORAGE (lowStorage=true) or CNS_RK3_CLASSIC */
    int32_t boundary_layer;      /* boundaryLayer (globals.h:33)                          */
    int32_t perturbed;           /* perturbed (globals.h:34)                              */
    int32_t forcing;             /* forcing: constant-mass-flux body force on z (globals.h:35) */
    int32_t periodic_x;          /* periodicX (globals.h:36)                              */
    int32_t nonuniform_x;        /* nonUniformX: tanh-stretched x (globals.h:37)          */
    double  stretch;             /* tanh stretching factor (globals.h:50)                 */
    double  twall_top, twall_bot;/* isothermal wall temperatures (globals.h:51-52)        */
    int32_t check_cfl;           /* checkCFLcondition: dt (and forcing) update period     */
    int32_t check_bulk;          /* checkBulk: bulk / kinetic-energy diagnostic period    */
    int32_t quirk_dissipation_y; /* 1: reproduce the reference's y viscous-dissipation
                                    term tau_yz*dv/dz (src/cuda_rhs.cu:175); 0: tau_yz*dw/dy */
    int32_t precision;           /* CNS_PREC_FP64, CNS_PREC_FP32_RHS or CNS_PREC_PAIR_RHS  */
    int32_t ndivz;               /* nDivZ (globals.h:58): accepted for compatibility, no effect */
    double  dpdz_init;           /* initial body force when forcing (cuda_utils.cu:69: 0.00372) */
    /* sponge constants (src/sponge.h:4-17) */
    double  sp_top_str, sp_top_len, sp_top_exp;
    double  sp_inl_str, sp_inl_len, sp_inl_exp;
    double  sp_out_str, sp_out_len, sp_out_exp;
    /* wall perturbation constants (src/perturbation.h:14-22) */
    int32_t pert_kc, pert_lp;
    double  pert_amp1, pert_amp2, pert_omega1_per_re, pert_omega2;
} cns_params;

typedef struct cns_solver cns_solver;

/* Fill *p with the values of the reference's src/globals.h / sponge.h / perturbation.h
 * defaults for everything that is not a grid size (grid set to 64^3 periodic TGV). */
CNS_API void        cns_default_params(cns_params* p);

/* Validate parameters without touching a device. Returns CNS_OK or CNS_ERR_INVALID. */
CNS_API int         cns_check_params(const cns_params* p);

/* Thread-local message describing the last failure on this thread ("" if none). */
CNS_API const char* cns_last_error(void);

/* Library version string. */
CNS_API const char* cns_version(void);

/* setDevice + setGPUParameters + initSolver (src/cuda_utils.cu:49-179,415-519):
 * builds the grid (src/init.cpp:32-92), coefficient tables and allocates the
 * device state on `device`. */
CNS_API int cns_create(const cns_params* p, int device, cns_solver** out);

/* clearSolver (src/cuda_utils.cu:521-595). NULL is accepted. */
CNS_API int cns_destroy(cns_solver* h);

/* Set the CUDA stream (a cudaStream_t cast to void*) for all work of this handle.
 * NULL selects the handle's own stream. */
CNS_API int cns_set_stream(cns_solver* h, void* stream);

/* Grid built by initGrid/derivGrid (src/init.cpp:32-92,258-277): x[mx], xp[mx]
 * (= 1/x'(xi)), xpp[mx] (= x''(xi)), y[my], z[mz]. Any pointer may be NULL. */
CNS_API int cns_get_grid(cns_solver* h, double* x, double* xp, double* xpp, double* y, double* z);

/* The same grid computed on the host from parameters alone (no device, no handle). */
CNS_API int cns_host_grid(const cns_params* p, double* x, double* xp, double* xpp, double* y, double* z);

/* calculateSponge (src/sponge.cu:83-240) from a 1D self-similar profile
 * (the reference's blasius1D/{x,r,u,w,e}Prof.bin): sponge strengths from the sponge
 * constants, reference fields by cubic-spline interpolation of the profile at
 * x/sqrt(1+z/Re). When `init_fields` is non-zero the state is also set to the
 * reference fields (restartFile < 0 in the reference). */
CNS_API int cns_set_sponge_profiles(cns_solver* h, int n, const double* xin, const double* rin,
                            const double* uin, const double* win, const double* ein,
                            int init_fields);

/* Direct form: sponge_x[mx], sponge_z[mz] and the reference fields r, u, w, rhoE
 * on the (x,z) plane, each mx*mz, index i + k*mx (src/sponge.h:36-37). u_ref and
 * w_ref are velocities; momentum references are formed as in copySpongeToDevice
 * (src/sponge.cu:57-61). */
CNS_API int cns_set_sponge(cns_solver* h, const double* sponge_x, const double* sponge_z,
                   const double* rref, const double* uref, const double* wref,
                   const double* eref);

/* copyField (src/cuda_utils.cu:299-370). direction 0: host -> device, followed by
 * the state recomputation (calcState). direction 1: device -> host. */
CNS_API int cns_copy_field(cns_solver* h, int direction, double* r, double* u, double* v,
                   double* w, double* e);

/* runSimulationLowStorage / runSimulation (src/cuda_main.cu:109-186, :44-107):
 * advance `nsteps` time steps. Every check_cfl steps (counted from the handle's
 * step counter) dt and, with forcing, the body force are recomputed on the device;
 * every check_bulk steps the bulk diagnostic is evaluated. The optional host
 * arrays par1, par2, time (length nsteps) receive, per step, the bulk diagnostics
 * (unforced: par1 = <u.u>, the reference's kinetic-energy diagnostic, and
 * par2 = <rho |u|^2>/2; forced: bulk velocity int(rho w)/int(rho) and int(rhoE);
 * NaN on steps without a diagnostic) and the simulation time after the step, as the
 * reference's dpar1/dpar2/dtime. Steps are replayed from a captured CUDA graph
 * (cns_set_graphs). */
CNS_API int cns_run(cns_solver* h, int nsteps, double* par1, double* par2, double* time);

/* Enable (default) or disable CUDA-graph replay of the time step in cns_run. The
 * reference launches every kernel from the host; no counterpart. */
CNS_API int cns_set_graphs(cns_solver* h, int enable);

/* One evaluation of calcRHS (src/cuda_main.cu:15-42) on the current state, copied to
 * the host: d(rho)/dt, d(rho u)/dt, d(rho v)/dt, d(rho w)/dt, d(rho E)/dt. */
CNS_API int cns_calc_rhs(cns_solver* h, double* rr, double* ru, double* rv, double* rw, double* re);

/* Current dt, body force dpdz and simulation time (device scalars dtC, dpdz,
 * time_on_GPU of the reference). Any pointer may be NULL. */
CNS_API int cns_get_scalars(cns_solver* h, double* dt, double* dpdz, double* time);

/* Override dt, dpdz, simulation time and the step counter (restart bookkeeping).
 * Negative step leaves the counter unchanged. */
CNS_API int cns_set_scalars(cns_solver* h, double dt, double dpdz, double time, int64_t step);

/* Time `nstages` Runge-Kutta stages (low-storage coefficients, the state advances) phase
 * by phase with CUDA events on the handle's stream. ms[0]: ghost fill of the stencil
 * inputs, ms[1]: velocity gradients + dilatation ghosts, ms[2]: the RHS + stage-update
 * kernel, which also recovers T, p, H, mu of the new state for the next stage; averages
 * per stage. No counterpart in the reference (it has no timers, src/main.cpp:71-75). */
CNS_API int cns_time_phases(cns_solver* h, int nstages, double* ms);

/* Number of CUDA kernels this handle has launched since creation. */
CNS_API int64_t cns_kernel_launches(const cns_solver* h);

/* Device bytes held by the handle. */
CNS_API int64_t cns_device_bytes(const cns_solver* h);

/* Plane profiles over (y, z) of the current state, the reference's calcAvgChan
 * (src/init.cpp:150-208, its prof.txt) evaluated on the device: out[q * mx + i] for
 * q = 0..10 = x, <rho>, <rho u>/<rho>, <rho v>/<rho>, <rho w>/<rho>, <rhoE>, and the
 * (y, z) means of (rho - <rho>)^2, (u - ~u)^2, (v - ~v)^2, (w - ~w)^2, (rhoE - <rhoE>)^2. */
CNS_API int cns_plane_stats(cns_solver* h, double* out);

/* Friction Reynolds number at the x = 0 wall of the current state, the reference's
 * printRes (src/init.cpp:210-256) on the device: the (y, z) mean of u_tau rho_w / mu_w,
 * u_tau = sqrt(mu_w |dw/dx| / rho_w), mu_w = 1^viscexp / Re, dw/dx at the first point at
 * the advective order from the interior values mirrored evenly about the wall. */
CNS_API int cns_friction_reynolds(cns_solver* h, double* ret);

/* Volume-averaged viscous dissipation and enstrophy of the current state, in FP64 from the
 * FP64 state (either precision mode): out[0] = < tau_ij du_i/dx_j >, tau_ij = mu (du_i/dx_j
 * + du_j/dx_i - 2/3 delta_ij theta), mu = T^viscexp / Re; out[1] = < |curl u|^2 >; means
 * with the cell volumes over the box, gradients as derVelX/Y/Z (src/calc_stress.cu:20-63)
 * at the viscous order. The reference computes neither (post-processing). */
CNS_API int cns_dissipation(cns_solver* h, double* out);

/* Stateless device reductions of a caller-owned state, the reference's calcTimeStep
 * (deviceCalcDt + hostReduceToMin, src/calc_stress.cu:122-160, src/cuda_math.cu:308-333)
 * and the volume integrals of calcPressureGrad / calcBulk (src/calc_stress.cu:98-201,
 * hostVolumeIntegral src/cuda_math.cu:335-359). Inputs are device pointers to contiguous
 * [k][j][i] FP64 fields of mx*my*mz points: rho, primitive u, v, w, rhoE and the dynamic
 * viscosity mu; dxv[mx] (device) the x cell widths, dy, dz the uniform y/z spacings.
 * out (device, 5 doubles): [0] CFL time step min(cfl / max(convective, viscous rate)),
 * [1] sum rho dV, [2] sum rho w dV, [3] sum rhoE dV, [4] sum |u|^2 dV, dV = dxv*dy*dz.
 * Like the reference, it allocates its scratch (5*mz doubles) with cudaMalloc per call;
 * work is issued on `stream` (a cudaStream_t, NULL = legacy default) and the call
 * returns after the stream has finished. */
CNS_API int cns_reduce_state(int mx, int my, int mz, const double* r, const double* u, const double* v,
                             const double* w, const double* e, const double* mu, const double* dxv, double dy,
                             double dz, double gam, double cfl, double* out, void* stream);

/* Allocation-free variant of cns_reduce_state; it has no counterpart in the reference.
 * For callers that may not call cudaMalloc: code whose device memory all belongs to
 * another allocator (a host framework's caching allocator) or to a fixed HBM budget
 * that a serving process divides among its simulations, and time-critical loops that
 * must not block in cudaMalloc/cudaFree (cudaFree waits for the whole device). Same
 * arguments and results as cns_reduce_state, but the per-plane partials live in a fixed
 * device array of 5 * CNS_NOALLOC_MAX_PLANES doubles (160 KiB, held by every GPU that
 * loads the library until the process exits) and the call neither allocates nor frees
 * memory nor synchronises: results are ready when `stream` reaches this point.
 * mz > CNS_NOALLOC_MAX_PLANES is rejected with CNS_ERR_INVALID. The first call on a
 * device looks up the array's device address (a one-time cudaGetSymbolAddress with that
 * device current); make that first call before any stream capture. After
 * cudaDeviceReset on a device the looked-up address is stale and later calls on that
 * device are invalid. All calls share the array: calls whose work overlaps on the GPU
 * race and must be serialised by the caller. */
#define CNS_NOALLOC_MAX_PLANES 4096
CNS_API int cns_reduce_state_noalloc(int mx, int my, int mz, const double* r, const double* u, const double* v,
                                     const double* w, const double* e, const double* mu, const double* dxv,
                                     double dy, double dz, double gam, double cfl, double* out, void* stream);

/* ---------------------------------------------------------------------------------------
 * Batched ensemble (no counterpart in the reference, which runs one simulation per
 * executable): many simulations of different grid sizes and physical parameters that
 * share the stencil orders, the precision and the Wray RK3 scheme advance together: one
 * persistent cooperative kernel launch per Runge-Kutta stage for the whole batch, or each
 * member's own step graph on one of CNS_BATCH_LANES concurrent streams (the execution
 * mode, chosen by cns_batch_tune), the step replayed from captured CUDA graphs. A member's
 * handle (cns_batch_member) takes per-member settings such as its sponge. Members keep
 * their own dt (CFL), body
 * force, bulk schedule, time and per-step logs. Membership may change between steps
 * (continuous batching); admission respects an optional HBM budget.
 * ------------------------------------------------------------------------------------- */
#define CNS_BATCH_MAX 256
typedef struct cns_batch cns_batch;

/* hbm_budget_bytes <= 0: no budget. */
CNS_API int cns_batch_create(int device, int precision, int stencil_size, int stencil_visc,
                             int64_t hbm_budget_bytes, cns_batch** out);
CNS_API int cns_batch_destroy(cns_batch* b);
CNS_API int cns_batch_set_stream(cns_batch* b, void* stream);
/* Admit a simulation with host initial fields ([k][j][i], as cns_copy_field);
 * max_steps sizes its per-step logs. CNS_ERR_OOM if the budget (or CNS_BATCH_MAX) would
 * be exceeded; the batch is unchanged then. */
CNS_API int cns_batch_add(cns_batch* b, const cns_params* p, const double* r, const double* u,
                          const double* v, const double* w, const double* e, int max_steps, int* id_out);
CNS_API int cns_batch_remove(cns_batch* b, int id);
/* The member's solver handle (for cns_set_sponge, cns_get_scalars, cns_copy_field(1) ...);
 * valid until the member is removed. NULL for an unknown id. */
CNS_API cns_solver* cns_batch_member(cns_batch* b, int id);
CNS_API int cns_batch_get_fields(cns_batch* b, int id, double* r, double* u, double* v, double* w, double* e);
/* First n per-step logs of a member (as cns_run's par1/par2/time) and its current dt. */
CNS_API int cns_batch_get_logs(cns_batch* b, int id, int n, double* par1, double* par2, double* time, double* dt);
CNS_API int cns_batch_member_steps(cns_batch* b, int id, int64_t* steps);
CNS_API int cns_batch_info(cns_batch* b, int* count, int64_t* points, int64_t* bytes, int64_t* launches);
/* Advance every member by nsteps steps. */
CNS_API int cns_batch_step(cns_batch* b, int nsteps);
/* Launch shape of the persistent stage kernel: 128 threads per block (the only shape; a work
 * unit is a 32 x 4 tile of an x-y plane), blocks per SM (clamped to the co-residency limit). */
CNS_API int cns_batch_set_shape(cns_batch* b, int threads, int blocks_per_sm);
CNS_API int cns_batch_get_shape(cns_batch* b, int* threads, int* blocks_per_sm);

/* Execution mode (no counterpart in the reference): CNS_BATCH_PERSISTENT advances all
 * members with one persistent cooperative launch per RK stage (launch shape as above);
 * CNS_BATCH_CONCURRENT advances each member through its own captured step graph on one
 * of up to CNS_BATCH_LANES streams, so the members' kernels overlap. cns_batch_tune
 * measures both and keeps the faster. */
#define CNS_BATCH_PERSISTENT 0
#define CNS_BATCH_CONCURRENT 1
#define CNS_BATCH_LANES 16
CNS_API int cns_batch_set_mode(cns_batch* b, int mode);
CNS_API int cns_batch_get_mode(cns_batch* b, int* mode);
/* Autotune the launch shape by timing `steps` steps per candidate on the current members
 * (the members advance); the choice is cached per precision, stencil orders and size
 * class. best_ms receives the best time per step (-1 when taken from the cache). */
CNS_API int cns_batch_tune(cns_batch* b, int steps, double* best_ms);

/* ---------------------------------------------------------------------------------------
 * Serving (no counterpart in the reference): a request loop for "advance N steps" solves
 * with continuous batching. Requests (parameters, initial fields, N) are submitted from
 * any thread; one worker thread owns a GPU batch, admits queued requests between steps
 * in arrival order while the HBM budget allows, advances all resident simulations one
 * step per tick and retires finished ones (fields copied to host memory, device memory
 * released). Latency = submit to result ready.
 * ------------------------------------------------------------------------------------- */
typedef struct cns_server cns_server;
#define CNS_REQ_QUEUED  0
#define CNS_REQ_RUNNING 1
#define CNS_REQ_DONE    2
#define CNS_REQ_FAILED  3
typedef struct cns_server_stats_t {
    int64_t completed, queued, running;   /* requests */
    int64_t batch_steps;                  /* batch steps taken by the worker */
    int64_t point_steps;                  /* grid points x steps advanced */
    double busy_seconds;                  /* first admission to last completion */
    double p50_s, p99_s, max_s;           /* latency percentiles of completed requests */
} cns_server_stats_t;

/* max_batch <= 0: up to CNS_BATCH_MAX resident simulations. */
CNS_API int cns_server_create(int device, int precision, int stencil_size, int stencil_visc,
                              int64_t hbm_budget_bytes, int max_batch, cns_server** out);
CNS_API int cns_server_destroy(cns_server* s);
/* Copies the initial fields; thread-safe. */
CNS_API int cns_server_submit(cns_server* s, const cns_params* p, const double* r, const double* u,
                              const double* v, const double* w, const double* e, int nsteps, int64_t* req_id);
CNS_API int cns_server_poll(cns_server* s, int64_t req_id, int* state, double* latency_s);
/* Blocks up to timeout_s for the result and copies the final fields (any may be NULL);
 * the request is forgotten afterwards. CNS_ERR_TIMEOUT if not finished in time. */
CNS_API int cns_server_wait(cns_server* s, int64_t req_id, double timeout_s, double* r, double* u,
                            double* v, double* w, double* e);
CNS_API int cns_server_stats(cns_server* s, cns_server_stats_t* st);

/* Failure-detection self test (no counterpart in the reference): one block waits at the
 * batch kernel's bounded grid barrier for a block that does not exist; the wait must give
 * up after spin_limit (1..2^20) polls. *timed_out = 1 when it did. Nothing hangs. */
CNS_API int cns_selftest_barrier_timeout(int device, long long spin_limit, int* timed_out);

/* Measurement utility with no counterpart in the reference: dependency-free FMA
 * throughput of the FP64 (fp64 = 1) or FP32 pipe on `device`, in TFLOP/s (FMA = 2),
 * over `iters` iterations of 8 independent chains per thread. It states the pipe
 * roofline next to the measured HBM bandwidth. */
CNS_API int cns_probe_fma_peak(int device, int fp64, int iters, double* tflops);

/* Self test with no counterpart in the reference: the solver's FP64 -> FP32 and FP32 ->
 * FP64 conversions, which run on the integer units, next to the hardware conversions on
 * the same inputs (n <= 2^28 values each; host arrays). The contract: bitwise equal,
 * except that magnitudes below 2^-126 become a zero of the same sign and NaN stays NaN. */
CNS_API int cns_selftest_convert(int device, const double* x, const float* y, long long n, float* f_alu, float* f_hw,
                                 double* d_alu, double* d_hw);

/* Self test with no counterpart in the reference: the solver's FP64 power for the
 * viscosity law (T^viscexp) next to the CUDA library pow on the same n <= 2^27 host
 * values. */
CNS_API int cns_selftest_pow(int device, const double* x, long long n, double a, double* fast, double* lib);

/* Self test with no counterpart in the reference: the solver's FP64 reciprocal (an FP32
 * seed r0 refined as r0 (1 + e + e^2), used for 1/rho in every stage update and state
 * recovery) next to the IEEE division 1.0 / x on the same n <= 2^27 host values. */
CNS_API int cns_selftest_rcp(int device, const double* x, long long n, double* fast, double* lib);

/* Self test with no counterpart in the reference: the pair arithmetic of
 * CNS_PREC_PAIR_RHS on n <= 2^24 host triples (a, b, c), each first split into its nearest
 * pair. out[(t * 15 + q) * 2 + {0, 1}] holds the two floats of result q of element t:
 * q = 0..2 the pairs of a, b, c; 3..6 a + b, a b, fma(a, b, c) and the compensated
 * accumulation c + a b; 7..10 the same four from the packed two-lane forms, lane 0 on
 * (a, b, c); 11..14 lane 1 on (b, c, a). */
CNS_API int cns_selftest_pair(int device, const double* a, const double* b, const double* c, long long n,
                              float* out);

#ifdef __cplusplus
}
#endif

#endif /* CNS_GB300_H_ */
