/*
 * mpgos.h - C-ABI of the GB300 ensemble explicit Runge-Kutta integrator.
 *
 * This is the boundary that replaces the host object of the reference,
 * class ProblemSolver in SourceCodes/SingleSystem_PerThread_Interface.cuh:117-208
 * (and the kernel launch it performs in Solve(), :1279-1285). Plain C types
 * only: opaque handles, pointers, sizes and int status codes.
 *
 * Two pieces meet at this ABI:
 *   - the runtime (libmpgos_runtime.so) owns device memory, pinned host
 *     buffers, the stream, CUDA graphs, timing and the autotuner;
 *   - a system plugin (libmpgos_<system>.so, or the user's own translation
 *     unit through the C++ drop-in header mpgos/SingleSystem_PerThread_Interface.cuh)
 *     holds the sm_103a kernels instantiated for one set of user device hooks
 *     (the PerThread_* templates of the reference, e.g.
 *     Tutorials_SingleSystem_PerThread/T1_Reference/Reference_SystemDefinition.cuh:6-76)
 *     and hands the runtime an mpgos_pt_kernels table.
 *
 * Error convention: every function returns MPGOS_OK (0) or a positive error
 * code; mpgos_last_error() returns a thread-local message for the last error.
 * The reference prints and calls exit(1) instead
 * (SingleSystem_PerThread_Interface.cuh:13-22, :566-581); the C++ drop-in
 * header restores that behaviour on top of these codes.
 */
#ifndef MPGOS_H
#define MPGOS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MPGOS_ABI_VERSION 2

/* ---- status codes ------------------------------------------------------ */
enum mpgos_status {
    MPGOS_OK              = 0,
    MPGOS_ERR_ARGUMENT    = 1, /* bad index, option, variable or value      */
    MPGOS_ERR_CUDA        = 2, /* a CUDA runtime call failed                */
    MPGOS_ERR_MEMORY      = 3, /* device or pinned host allocation failed   */
    MPGOS_ERR_SHAPE       = 4, /* kernel table does not match the request   */
    MPGOS_ERR_UNSUPPORTED = 5  /* mode or feature not compiled in           */
};

/* ---- Algorithms (SingleSystem_PerThread_Interface.cuh:33) --------------- */
enum mpgos_algorithm { MPGOS_RK4 = 0, MPGOS_RKCK45 = 1 };

/* ---- ListOfVariables (SingleSystem_PerThread_Interface.cuh:35-47) -------- */
enum mpgos_variable {
    MPGOS_ALL                       = 0,
    MPGOS_TIME_DOMAIN               = 1,  /* [2][NT]                 */
    MPGOS_ACTUAL_STATE              = 2,  /* [SD][NT]                */
    MPGOS_ACTUAL_TIME               = 3,  /* [NT]                    */
    MPGOS_CONTROL_PARAMETERS        = 4,  /* [NCP][NT]               */
    MPGOS_SHARED_PARAMETERS         = 5,  /* [NSP]                   */
    MPGOS_INTEGER_SHARED_PARAMETERS = 6,  /* [NISP] (int32)          */
    MPGOS_ACCESSORIES               = 7,  /* [NA][NT]                */
    MPGOS_INTEGER_ACCESSORIES       = 8,  /* [NIA][NT] (int32)       */
    MPGOS_DENSE_OUTPUT              = 9,  /* index + time + state    */
    MPGOS_DENSE_INDEX               = 10, /* [NT] (int32)            */
    MPGOS_DENSE_TIME                = 11, /* [NDO][NT]               */
    MPGOS_DENSE_STATE               = 12, /* [NDO][SD][NT]           */
    /* extensions (no counterpart in the reference) */
    MPGOS_STATUS                    = 32, /* [NT] int32 bit flags of the last Solve  */
    MPGOS_ACCEPTED_STEPS            = 33, /* [NT] int32, accepted steps, last Solve  */
    MPGOS_REJECTED_STEPS            = 34  /* [NT] int32, rejected attempts, last Solve */
};

/* ---- ListOfSolverOptions (SingleSystem_PerThread_Interface.cuh:49-62) ---- */
enum mpgos_option {
    MPGOS_THREADS_PER_BLOCK            = 0,
    MPGOS_INITIAL_TIME_STEP            = 1,
    MPGOS_ACTIVE_NUMBER_OF_THREADS     = 2,
    MPGOS_MAXIMUM_TIME_STEP            = 3,
    MPGOS_MINIMUM_TIME_STEP            = 4,
    MPGOS_TIME_STEP_GROW_LIMIT         = 5,
    MPGOS_TIME_STEP_SHRINK_LIMIT       = 6,
    MPGOS_RELATIVE_TOLERANCE           = 7,  /* indexed by component  */
    MPGOS_ABSOLUTE_TOLERANCE           = 8,  /* indexed by component  */
    MPGOS_EVENT_TOLERANCE              = 9,  /* indexed by event      */
    MPGOS_EVENT_DIRECTION              = 10, /* indexed by event      */
    MPGOS_DENSE_OUTPUT_MINIMUM_TIME_STEP = 11,
    MPGOS_DENSE_OUTPUT_SAVE_FREQUENCY  = 12,
    MPGOS_PREFER_SHARED_MEMORY         = 13,
    /* extensions */
    MPGOS_KERNEL_MODE                  = 32, /* MPGOS_MODE_* bit set             */
    MPGOS_MAXIMUM_ATTEMPTS             = 33, /* step attempts per instance and launch */
    MPGOS_INSTANCES_PER_THREAD         = 34, /* static mapping: instances each lane integrates in turn (grid stride) */
    MPGOS_WARP_RECONVERGE              = 35, /* 1: the integrating lanes of a warp reconverge once per step attempt
                                                (a warp ballot; pays where lanes diverge: events, uneven
                                                accept/reject); 0: leave it to the compiler. Default 1 for
                                                systems with events, else 0; the autotuner tries both. */
    MPGOS_OUTLINE_RHS                  = 36, /* DF_STAGE: 1 = the right-hand side as one out-of-line function
                                                (its code once in the kernel instead of once per stage; pays
                                                for large right-hand sides that overflow the instruction
                                                cache), 0 = inlined (default); results are identical. The
                                                autotuner tries both for double-float kernels. */
    MPGOS_WORK_ORDER                   = 37  /* 1: every launch integrates the instances longest first by
                                                the step attempts of the previous launch (a counting sort on
                                                the device before the launch; both mappings: the persistent
                                                queue and the static lanes take instances in that order),
                                                so the last wave of an uneven launch is short and a warp's
                                                lanes hold instances of similar length; 0: index order
                                                (default). Each instance's results are identical. */
};

/* ---- kernel modes (extensions) -----------------------------------------
 * PLAIN        reference arithmetic: one instance per thread, static grid,
 *              controller with FP64 pow/div exactly as
 *              SingleSystem_PerThread_ExplicitRungeKutta_ErrorControllers.cuh:23-85.
 * FAST_CONTROL step-size factor from FP32 log2/exp2 of the tolerance ratio and
 *              integer-pipe compares on FP64 bit patterns; accept/reject
 *              decisions are unchanged, the new step size differs from the
 *              FP64 pow by about 1e-7 relative.
 * PERSISTENT   one resident grid; every lane pulls the next instance from a
 *              device work counter when its instance finishes.
 * FP32_STAGE   right-hand side and stage sums in FP32; state update, time,
 *              error norm, step control and events in FP64 (RKCK45 only).
 * CHOSEN       FAST_CONTROL | PERSISTENT.
 */
#define MPGOS_MODE_PLAIN        0
#define MPGOS_MODE_FAST_CONTROL 1
#define MPGOS_MODE_PERSISTENT   2
#define MPGOS_MODE_FP32_STAGE   4
/* DF_STAGE: every per-instance quantity of the FP64 scheme in double-float
 * arithmetic (pairs of floats, ~48 significant bits) on the FP32 pipe: RKCK45
 * with a log-domain step-size factor, RK4 on the reference's FP64 time grid
 * (identical step counts); results agree with the FP64 kernels to ~1e-13
 * relative on non-chaotic instances. Exclusive with FP32_STAGE; FAST_CONTROL
 * is implied. */
#define MPGOS_MODE_DF_STAGE     16
/* SPLIT: the precision split of the FP32-stage mode with double-float stages:
 * the right-hand side (the user's hook instantiated for double-float) and the
 * stage sums in double-float on the FP32 pipe; the state update
 * x + dt * sum b_i k_i, the time, the step size, the error estimate and norm,
 * the accept test, the step-size factor (to FP64 accuracy), the event
 * functions, the secant step toward events, dense output and every other hook
 * in FP64. RKCK45 and RK4 (RK4 on the reference's FP64 time grid). Exclusive
 * with FP32_STAGE and DF_STAGE; FAST_CONTROL is implied. The coupled solver
 * has it too: the unit right-hand sides, the coupling values and terms and
 * the stage sums in double-float; the warp's accept test, minimum ratio and
 * step factor (safety factor 0.8) in FP64. */
#define MPGOS_MODE_SPLIT        128
#define MPGOS_MODE_CHOSEN       (MPGOS_MODE_FAST_CONTROL | MPGOS_MODE_PERSISTENT)

/* ---- per-instance status flags (MPGOS_STATUS), extensions --------------
 * The reference reports these conditions with device printf only
 * (SingleSystem_PerThread_ExplicitRungeKutta_ErrorControllers.cuh:15,66,73,
 *  SingleSystem_PerThread_EventHandling.cuh:38). */
#define MPGOS_INSTANCE_OK               0
#define MPGOS_INSTANCE_NONFINITE        1  /* stopped: state not finite            */
#define MPGOS_INSTANCE_MINIMUM_STEP     2  /* warning: continued at minimum step    */
#define MPGOS_INSTANCE_EVENT_OMITTED    4  /* warning: event step below minimum     */
#define MPGOS_INSTANCE_ATTEMPT_LIMIT    8  /* stopped: MPGOS_MAXIMUM_ATTEMPTS hit   */
#define MPGOS_INSTANCE_TAPE_OVERFLOW   16  /* adjoint: more accepted steps than the tape holds */
#define MPGOS_INSTANCE_RANGE           32  /* warning (DF_STAGE, SPLIT): a value the double-float
                                              arithmetic holds left float's exponent range
                                              (|v| >= 2^128 or 0 < |v| < 2^-126); it loses
                                              precision or overflows there */

/* ---- kernel table handed from a system plugin to the runtime ----------- */

/* Compile-time shape of a system plugin (template parameters of the
 * reference's ProblemSolver, SingleSystem_PerThread_Interface.cuh:117). */
typedef struct mpgos_pt_shape {
    int32_t sd, ncp, nsp, nisp, ne, na, nia;
    int32_t algorithm;       /* mpgos_algorithm             */
    int32_t precision_bytes; /* 8 = double, 4 = float      */
    int32_t modes;           /* MPGOS_MODE_* bits compiled  */
} mpgos_pt_shape;

/* Everything one launch needs. Mirrors the by-value kernel arguments of the
 * reference (Struct_ThreadConfiguration, Struct_GlobalVariables,
 * Struct_SharedMemoryUsage, Struct_SolverOptions,
 * SingleSystem_PerThread_Interface.cuh:72-115), plus the extensions. Device
 * pointers; floating-point arrays are in the table's precision. */
typedef struct mpgos_pt_launch {
    int64_t nt;           /* instances allocated (SoA stride)       */
    int64_t n_active;     /* instances integrated: 0 .. n_active-1  */
    int32_t ndo;          /* dense-output slots per instance        */
    int32_t mode;         /* MPGOS_MODE_* bits                      */
    int32_t prefer_shared;
    int32_t dense_save_frequency;
    int64_t max_attempts;
    double  initial_dt, max_dt, min_dt, grow_limit, shrink_limit, dense_min_dt;

    void*          time_domain;
    void*          actual_state;
    void*          actual_time;
    void*          control_parameters;
    const void*    shared_parameters;
    const int32_t* integer_shared_parameters;
    void*          accessories;
    int32_t*       integer_accessories;
    const void*    relative_tolerance;
    const void*    absolute_tolerance;
    const void*    event_tolerance;
    const int32_t* event_direction;
    int32_t*       dense_index;
    void*          dense_time;
    void*          dense_state;
    int32_t*       status;          /* [NT] or NULL */
    int32_t*       accepted_steps;  /* [NT] or NULL */
    int32_t*       rejected_steps;  /* [NT] or NULL */
    uint32_t*      work_counter;    /* PERSISTENT: one zeroed counter */
    const int32_t* instance_order;  /* [n_active] instance of each work item, or NULL (identity) */
} mpgos_pt_launch;

/* Adjoint tape (extension): frozen step sizes and state checkpoints of a
 * recorded forward pass, device pointers, FP64. */
typedef struct mpgos_pt_tape {
    int32_t  segment;    /* accepted steps between checkpoints (<= 64)      */
    int32_t  max_steps;  /* tape capacity in accepted steps per instance    */
    double*  dt;         /* [max_steps][NT]                                 */
    double*  ckpt_x;     /* [max_steps/segment + 1][SD][NT]                 */
    double*  ckpt_t;     /* [max_steps/segment + 1][NT]                     */
    int32_t* n_steps;    /* [NT] accepted steps recorded                    */
} mpgos_pt_tape;

typedef struct mpgos_pt_kernels {
    int32_t        abi_version;     /* MPGOS_ABI_VERSION */
    mpgos_pt_shape shape;
    const char*    name;
    /* Launch on the given cudaStream_t; returns a cudaError_t value. */
    int (*launch)(const mpgos_pt_launch* args, int grid, int block, size_t dynamic_smem, void* stream);
    /* Resident blocks per SM for (mode, block, dynamic smem); cudaError_t. */
    int (*occupancy)(int32_t mode, int block, size_t dynamic_smem, int* blocks_per_sm);
    /* Adjoint (NULL when not compiled): forward launch that records the tape,
     * and the reverse launch (one instance per thread) computing
     * dL/dx(t0) [SD][NT] and dL/dcPAR [NCP][NT] from dL/dx(T) [SD][NT]. */
    int (*launch_record)(const mpgos_pt_launch* args, const mpgos_pt_tape* tape, int grid, int block,
                         size_t dynamic_smem, void* stream);
    int (*launch_adjoint)(const mpgos_pt_launch* args, const mpgos_pt_tape* tape, const double* dL_dxT,
                          double* dL_dx0, double* dL_dp, int grid, int block, size_t dynamic_smem, void* stream);
    /* Dense-output interpolation at n_times requested times (device arrays;
     * out [n_times][SD][NT], FP64), one instance per thread. */
    int (*dense_interpolate)(const mpgos_pt_launch* args, const double* times, int32_t n_times, double* out,
                             int grid, int block, size_t dynamic_smem, void* stream);
} mpgos_pt_kernels;

/* ---- solver object (ProblemSolver, SingleSystem_PerThread_Interface.cuh:117-208) */
typedef struct mpgos_pt_solver mpgos_pt_solver;

/* ProblemSolver(int device), :309-518: stream, event, pinned host + device
 * buffers sized for nt instances and ndo dense-output slots; defaults of
 * :475-496 (tolerances 1e-8, event tolerance 1e-6, direction 0). */
int mpgos_pt_create(const mpgos_pt_kernels* kernels, int64_t nt, int32_t ndo,
                    int device, mpgos_pt_solver** out);
/* ~ProblemSolver, :521-555. */
int mpgos_pt_destroy(mpgos_pt_solver* solver);
/* Compiled shape, instance count and dense slots of a solver. */
int mpgos_pt_get_shape(const mpgos_pt_solver* solver, mpgos_pt_shape* shape,
                       int64_t* nt, int32_t* ndo);

/* SolverOption(option, value) and SolverOption(option, index, value),
 * :611-703. index is ignored by the non-indexed options. Tolerance and event
 * options are pushed to the device immediately, as :679-694 do. */
int mpgos_pt_set_option(mpgos_pt_solver* solver, int32_t option, int32_t index, double value);
int mpgos_pt_get_option(const mpgos_pt_solver* solver, int32_t option, int32_t index, double* value);

/* Pinned host buffer of a variable (the h_* arrays of :399-409) and its
 * element count. SetHost/GetHost (:706-1080) become plain stores and loads
 * at index pid + serial*NT (dense state: pid + comp*NT + step*NT*SD). */
int mpgos_pt_host_buffer(mpgos_pt_solver* solver, int32_t variable, void** ptr, int64_t* count);
/* Device buffer of a variable (for callers that keep data resident in HBM). */
int mpgos_pt_device_buffer(mpgos_pt_solver* solver, int32_t variable, void** ptr, int64_t* count);

/* SynchroniseFromHostToDevice / SynchroniseFromDeviceToHost, :833-965.
 * Asynchronous on the solver's stream. */
int mpgos_pt_sync_h2d(mpgos_pt_solver* solver, int32_t variable);
int mpgos_pt_sync_d2h(mpgos_pt_solver* solver, int32_t variable);

/* Solve(), :1279-1285: one asynchronous launch on the solver's stream. The
 * step size restarts from InitialTimeStep on every launch, as
 * SingleSystem_PerThread_Solver.cuh:138-139 does. */
int mpgos_pt_solve(mpgos_pt_solver* solver);
/* n_phases consecutive Solve() calls, captured once into a CUDA graph and
 * replayed (extension). Bit-identical to n_phases calls of mpgos_pt_solve. If
 * stream_accessory >= 0, the accessory column stream_accessory is copied after
 * every phase into the device buffer phase_output[phase][NT]. */
int mpgos_pt_solve_phases(mpgos_pt_solver* solver, int32_t n_phases,
                          int32_t stream_accessory, void* phase_output);

/* InsertSynchronisationPoint / SynchroniseSolver / SynchroniseDevice,
 * :1288-1312. */
int mpgos_pt_insert_sync_point(mpgos_pt_solver* solver);
int mpgos_pt_sync_solver(mpgos_pt_solver* solver);
int mpgos_pt_sync_device(mpgos_pt_solver* solver);

/* Stream of the solver as a cudaStream_t (extension). */
int mpgos_pt_stream(mpgos_pt_solver* solver, void** stream);

/* Launch configuration the next Solve() will use (extension). */
int mpgos_pt_launch_config(mpgos_pt_solver* solver, int* grid, int* block, int32_t* mode);

/* Time with CUDA events on the solver's stream (extension): start, then stop
 * returns the elapsed milliseconds after synchronising the stop event. */
int mpgos_pt_timer_start(mpgos_pt_solver* solver);
int mpgos_pt_timer_stop(mpgos_pt_solver* solver, float* milliseconds);

/* Autotuner (extension): times one Solve() per candidate (block size x
 * mapping: static with 1, 2 or 4 instances per thread, or persistent x
 * placement of the shared parameters: shared memory or global loads, where the
 * system has any x, for double-float kernels, the right-hand side inlined or
 * out of line; then the warp reconvergence ballot on and off at the best of
 * those) on a scratch copy of the current device state,
 * restores the state, keeps the fastest configuration and, if cache_path is
 * not NULL, records it in a JSON cache keyed by system, shape, NT and GPU.
 * `arithmetic` fixes the arithmetic the candidates share: 0 the reference's,
 * MPGOS_MODE_SPLIT the precision split, MPGOS_MODE_DF_STAGE double-float
 * stages, any other non-zero value FAST_CONTROL (each where compiled, else
 * the reference's). */
int mpgos_pt_autotune(mpgos_pt_solver* solver, int32_t arithmetic, const char* cache_path);

/* Device-side checkpoint of every array a launch writes (time domain, state,
 * time, control parameters, accessories, dense output) and restore of it
 * (extension). The reference keeps the state only implicitly in the object
 * between Solve() calls (SingleSystem_PerThread_Solver.cuh:117-137, :414-435);
 * this makes a resumable snapshot explicit. Asynchronous on the stream. */
int mpgos_pt_checkpoint_save(mpgos_pt_solver* solver);
int mpgos_pt_checkpoint_restore(mpgos_pt_solver* solver);

/* Discrete adjoint (extension, no counterpart in the reference).
 * mpgos_pt_solve_record: one Solve() that also records the tape (every
 * accepted step size, a checkpoint every `segment` accepted steps; capacity
 * max_steps accepted steps per instance, device memory owned by the solver).
 * mpgos_pt_adjoint: reverse pass over the recorded tape. Device pointers,
 * FP64: dL_dxT [SD][NT] in, dL_dx0 [SD][NT] and dL_dp [NCP][NT] out; the
 * gradient of the discrete map with the recorded step sequence frozen.
 * Under MPGOS_MODE_DF_STAGE both passes compute in double-float (the tape
 * stays FP64: a double-float value is a double exactly); under
 * MPGOS_MODE_SPLIT the recording runs the split kernel and the reverse pass
 * computes in double-float; otherwise both in FP64.
 * The reverse arithmetic follows the mode set when mpgos_pt_adjoint is
 * called, so an FP64 tape can be reversed in double-float.
 * Instances whose step count exceeded the tape get MPGOS_INSTANCE_TAPE_OVERFLOW
 * in MPGOS_STATUS and no gradient. Asynchronous on the solver's stream. */
int mpgos_pt_solve_record(mpgos_pt_solver* solver, int32_t max_steps, int32_t segment);
int mpgos_pt_adjoint(mpgos_pt_solver* solver, const double* dL_dxT, double* dL_dx0, double* dL_dp);
/* Device pointers and sizes of the recorded tape (read-only view). */
int mpgos_pt_tape_info(const mpgos_pt_solver* solver, mpgos_pt_tape* tape);

/* Dense-output interpolation (extension; the reference stores the accepted
 * points only, SingleSystem_PerThread_DenseOutput.cuh:5-58): for every active
 * instance and each of the n_times requested times (device array, any order),
 * the cubic Hermite polynomial through the two stored points that bracket the
 * time, with the right-hand side at those points as slopes. Reads the device
 * copy of the dense output (a Solve with NDO > 0 before it); out is a device
 * array [n_times][SD][NT] in FP64 (instances past ActiveNumberOfThreads are
 * not written). Times outside an instance's stored range give NaN.
 * Asynchronous on the solver's stream. */
int mpgos_pt_dense_interpolate(mpgos_pt_solver* solver, const double* times, int32_t n_times, double* out);

/* mpgos_pt_solve_record without device allocation (no counterpart in the
 * reference): records the same tape as mpgos_pt_solve_record, bit for bit, into
 * a file-scope static device array of MPGOS_STATIC_TAPE_BYTES held by the
 * runtime library, instead of buffers it cudaMalloc's. No cudaMalloc, cudaFree
 * or other allocating call is made; the per-instance step counts are cleared
 * with cudaMemsetAsync on the solver's stream. A tape larger than
 * MPGOS_STATIC_TAPE_BYTES (dt: max_steps x NT doubles, checkpoints:
 * (max_steps / segment + 1) x (SD + 1) x NT doubles, counts: NT ints, each part
 * rounded up to 256 bytes) is rejected with MPGOS_ERR_ARGUMENT and a message.
 * mpgos_pt_adjoint and mpgos_pt_tape_info then read this tape until the next
 * mpgos_pt_solve_record. There is one such array per device and process:
 * overlapping calls (two solvers, or a second call before the first's reverse
 * pass has finished on the stream) race on it. The array is reserved when
 * the runtime's device module loads: mpgos_pt_create looks up its address
 * (cudaGetSymbolAddress) on every device it creates a solver on, so the
 * 16 MiB are taken at start-up, before a serving process's memory pool
 * reserves the free HBM. The recording and reverse kernels load lazily at
 * their first launch (CUDA's module loading takes a little device memory
 * then), so make one warm-up call at start-up, before any stream capture;
 * later calls take no device memory. The cached address belongs to the
 * device's primary context: after cudaDeviceReset this entry point must not
 * be used. */
#define MPGOS_STATIC_TAPE_BYTES (16u * 1024u * 1024u)
int mpgos_pt_solve_record_static(mpgos_pt_solver* solver, int32_t max_steps, int32_t segment);

/* Measured FMA throughput of the device (extension, no counterpart in the
 * reference): independent fused multiply-add chains in FP64
 * (precision_bytes 8) or FP32 (4) on every SM, timed with CUDA events.
 * Writes FLOP/s (one FMA = 2 FLOP). Used as the roofline denominator of the
 * FP64-pipe-bound kernels. */
int mpgos_probe_fma_peak(int device, int32_t precision_bytes, double* flops_per_second);

/* Double-float math probe (extension, for tests): evaluates one DF_STAGE
 * operation with the device build of the double-float arithmetic on n
 * argument pairs (host arrays a, b, each converted to double-float), writing
 * the result's two floats as doubles to out[2i] (hi) and out[2i + 1] (lo).
 * The SPLIT-mode operations take a and b as doubles: MPGOS_DF_SPLIT converts a
 * to double-float on the integer pipe (hi, lo out); MPGOS_DF_ROOT5 / ROOT4
 * give the split controller's (a / b)^(1/5) / (a / b)^(1/4) (FP32 estimate,
 * FP64 correction) in out[2i] and 0 in out[2i + 1]. */
enum mpgos_df_op {
    MPGOS_DF_EXP = 0, MPGOS_DF_LOG = 1, MPGOS_DF_POW = 2, MPGOS_DF_SIN = 3, MPGOS_DF_COS = 4,
    MPGOS_DF_SQRT = 5, MPGOS_DF_DIV = 6, MPGOS_DF_MUL = 7, MPGOS_DF_ADD = 8,
    MPGOS_DF_POW_INT = 9, /* pow(a, (int)b) */
    MPGOS_DF_SINPI = 10, MPGOS_DF_COSPI = 11,  /* the two results of sincospi(a) */
    MPGOS_DF_SPLIT = 12, MPGOS_DF_ROOT5 = 13, MPGOS_DF_ROOT4 = 14
};
int mpgos_probe_df_math(int device, int32_t op, int64_t n, const double* a, const double* b, double* out);

/* Thread-local message of the last failing call ("" if none). */
const char* mpgos_last_error(void);

/* Runtime ABI version (MPGOS_ABI_VERSION). */
int mpgos_abi_version(void);

/* =========================================================================
 * Coupled per-block solver (CoupledSystems_PerBlock_Interface.cuh:135-248):
 * NS systems of UPS coupled units. Unit-scope arrays are [field][NS*UPS]
 * with unit u of system s at s*UPS + u, system-scope arrays [field][NS]; the
 * coupling matrix is stored as the reference stores it for its (CBW, CCI)
 * (CoupledSystems_PerBlock_Interface.cuh:426-438, :993-1080).
 * ========================================================================= */

/* ListOfVariables of the coupled interface (CoupledSystems_PerBlock_Interface.cuh:33-52). */
enum mpgos_cb_variable {
    MPGOS_CB_ALL = 0, MPGOS_CB_TIME_DOMAIN = 1, MPGOS_CB_ACTUAL_TIME = 2, MPGOS_CB_ACTUAL_STATE = 3,
    MPGOS_CB_UNIT_PARAMETERS = 4, MPGOS_CB_SYSTEM_PARAMETERS = 5, MPGOS_CB_GLOBAL_PARAMETERS = 6,
    MPGOS_CB_INTEGER_GLOBAL_PARAMETERS = 7, MPGOS_CB_UNIT_ACCESSORIES = 8, MPGOS_CB_INTEGER_UNIT_ACCESSORIES = 9,
    MPGOS_CB_SYSTEM_ACCESSORIES = 10, MPGOS_CB_INTEGER_SYSTEM_ACCESSORIES = 11, MPGOS_CB_COUPLING_MATRIX = 12,
    MPGOS_CB_COUPLING_STRENGTH = 13, MPGOS_CB_COUPLING_INDEX = 14, MPGOS_CB_DENSE_OUTPUT = 15,
    MPGOS_CB_DENSE_INDEX = 16, MPGOS_CB_DENSE_TIME = 17, MPGOS_CB_DENSE_STATE = 18,
    /* extensions: per system, last Solve */
    MPGOS_CB_STATUS = 32, MPGOS_CB_ACCEPTED_STEPS = 33, MPGOS_CB_REJECTED_STEPS = 34
};

/* DF_STAGE keeps the coupling matrices in shared memory as double-floats when
 * they take at most this many bytes (NC x matrix_entries x 8), else reads a
 * double-float copy in global memory; fixed per system shape, so the kernel
 * knows at compile time which memory it reads. */
#define MPGOS_CB_DF_SHARED_MATRIX_BYTES (160 * 1024)

/* ListOfSolverOptions of the coupled interface (CoupledSystems_PerBlock_Interface.cuh:53-66). */
enum mpgos_cb_option {
    MPGOS_CB_INITIAL_TIME_STEP = 0, MPGOS_CB_ACTIVE_SYSTEMS = 1, MPGOS_CB_MAXIMUM_TIME_STEP = 2,
    MPGOS_CB_MINIMUM_TIME_STEP = 3, MPGOS_CB_TIME_STEP_GROW_LIMIT = 4, MPGOS_CB_TIME_STEP_SHRINK_LIMIT = 5,
    MPGOS_CB_RELATIVE_TOLERANCE = 6, MPGOS_CB_ABSOLUTE_TOLERANCE = 7, MPGOS_CB_EVENT_TOLERANCE = 8,
    MPGOS_CB_EVENT_DIRECTION = 9, MPGOS_CB_DENSE_OUTPUT_SAVE_FREQUENCY = 10,
    MPGOS_CB_DENSE_OUTPUT_MINIMUM_TIME_STEP = 11, MPGOS_CB_SHARED_GLOBAL_VARIABLES = 12,
    MPGOS_CB_SHARED_COUPLING_MATRICES = 13,
    /* extensions */
    MPGOS_CB_KERNEL_MODE = 32,          /* PERSISTENT, and DF_STAGE or SPLIT */
    MPGOS_CB_MAXIMUM_ATTEMPTS = 33,     /* step attempts per system         */
    MPGOS_CB_WARPS_PER_BLOCK = 34       /* systems per CTA (one per warp)   */
};

typedef struct mpgos_cb_shape {
    int32_t ups, ud, nc, cbw, cci, nup, nsp, ngp, nigp, nua, niua, nsa, nisa, ne;
    int32_t algorithm, precision_bytes;
    int32_t matrix_entries;  /* stored entries of one coupling matrix */
} mpgos_cb_shape;

typedef struct mpgos_cb_launch {
    int64_t ns, n_active;
    int32_t ndo, mode, shared_global, shared_coupling, dense_save_frequency, reserved;
    int64_t max_attempts;
    double  initial_dt, max_dt, min_dt, grow_limit, shrink_limit, dense_min_dt;
    void*          time_domain;                 /* [2][NS]        */
    void*          actual_time;                 /* [NS]           */
    void*          system_parameters;           /* [NSP][NS]      */
    void*          system_accessories;          /* [NSA][NS]      */
    int32_t*       integer_system_accessories;  /* [NISA][NS]     */
    void*          coupling_strength;           /* [NC][NS]       */
    int32_t*       dense_index;                 /* [NS]           */
    void*          dense_time;                  /* [NDO][NS]      */
    void*          actual_state;                /* [UD][NS*UPS]   */
    void*          unit_parameters;             /* [NUP][NS*UPS]  */
    void*          unit_accessories;            /* [NUA][NS*UPS]  */
    int32_t*       integer_unit_accessories;    /* [NIUA][NS*UPS] */
    void*          dense_state;                 /* [NDO][UD][NS*UPS] */
    const void*    global_parameters;           /* [NGP]          */
    const int32_t* integer_global_parameters;   /* [NIGP]         */
    const void*    coupling_matrix;             /* [NC][matrix_entries] */
    const int32_t* coupling_index;              /* [NC]           */
    const void*    relative_tolerance;          /* [UD]           */
    const void*    absolute_tolerance;          /* [UD]           */
    const void*    event_tolerance;             /* [NE]           */
    const int32_t* event_direction;             /* [NE]           */
    int32_t*       status;                      /* [NS]           */
    int32_t*       accepted_steps;              /* [NS]           */
    int32_t*       rejected_steps;              /* [NS]           */
    uint32_t*      work_counter;
    /* DF_STAGE with the coupling matrices too large for shared memory: their
     * double-float copy (pairs of floats, same layout), else NULL */
    const void*    coupling_matrix_df;
} mpgos_cb_launch;

typedef struct mpgos_cb_kernels {
    int32_t        abi_version;
    mpgos_cb_shape shape;
    const char*    name;
    int (*launch)(const mpgos_cb_launch* args, int grid, int block, size_t dynamic_smem, void* stream);
    int (*occupancy)(int32_t mode, int block, size_t dynamic_smem, int* blocks_per_sm);
    size_t (*dynamic_smem)(int warps_per_block, int shared_global, int shared_coupling);
    /* discrete adjoint (NULL where not compiled): the recording forward launch,
     * the reverse launch and its dynamic shared memory (FP64, or double-float
     * when `mode` has MPGOS_MODE_DF_STAGE) */
    int (*launch_record)(const mpgos_cb_launch* args, const mpgos_pt_tape* tape, int grid, int block,
                         size_t dynamic_smem, void* stream);
    int (*launch_adjoint)(const mpgos_cb_launch* args, const mpgos_pt_tape* tape, const double* dL_dxT,
                          double* dL_dx0, double* dL_dsp, int grid, int block, size_t dynamic_smem, void* stream);
    size_t (*adjoint_smem)(int warps_per_block, int32_t mode);
    int (*adjoint_occupancy)(int32_t mode, int block, size_t dynamic_smem, int* blocks_per_sm);
} mpgos_cb_kernels;

typedef struct mpgos_cb_solver mpgos_cb_solver;

/* ProblemSolver(int) / ~ProblemSolver of the coupled interface. */
int mpgos_cb_create(const mpgos_cb_kernels* kernels, int64_t ns, int32_t ndo, int device, mpgos_cb_solver** out);
int mpgos_cb_destroy(mpgos_cb_solver* solver);
int mpgos_cb_get_shape(const mpgos_cb_solver* solver, mpgos_cb_shape* shape, int64_t* ns, int32_t* ndo);
/* SolverOption (CoupledSystems_PerBlock_Interface.cuh:760-860). */
int mpgos_cb_set_option(mpgos_cb_solver* solver, int32_t option, int32_t index, double value);
/* Pinned host / device buffer of a variable and its element count. */
int mpgos_cb_host_buffer(mpgos_cb_solver* solver, int32_t variable, void** ptr, int64_t* count);
int mpgos_cb_device_buffer(mpgos_cb_solver* solver, int32_t variable, void** ptr, int64_t* count);
/* SynchroniseFromHostToDevice / SynchroniseFromDeviceToHost. */
int mpgos_cb_sync_h2d(mpgos_cb_solver* solver, int32_t variable);
int mpgos_cb_sync_d2h(mpgos_cb_solver* solver, int32_t variable);
/* Solve() (CoupledSystems_PerBlock_Interface.cuh:1947-1966): one launch. */
int mpgos_cb_solve(mpgos_cb_solver* solver);
int mpgos_cb_insert_sync_point(mpgos_cb_solver* solver);
int mpgos_cb_sync_solver(mpgos_cb_solver* solver);
int mpgos_cb_timer_start(mpgos_cb_solver* solver);
int mpgos_cb_timer_stop(mpgos_cb_solver* solver, float* milliseconds);
int mpgos_cb_stream(mpgos_cb_solver* solver, void** stream);
int mpgos_cb_checkpoint_save(mpgos_cb_solver* solver);
int mpgos_cb_checkpoint_restore(mpgos_cb_solver* solver);
/* Discrete adjoint of the coupled solver (extension, no counterpart in the
 * reference), FP64 tables; under MPGOS_MODE_DF_STAGE the recording and the
 * reverse pass compute in double-float (the tape stays FP64), and the reverse
 * arithmetic follows the mode set when mpgos_cb_adjoint is called.
 * mpgos_cb_solve_record: one Solve() that also
 * records the tape (every accepted step size of every system, the time and
 * every unit's state every `segment` accepted steps; capacity max_steps per
 * system; device memory owned by the solver). mpgos_cb_adjoint: reverse pass;
 * device pointers, FP64: dL_dxT [UD][NS*UPS] in, dL_dx0 [UD][NS*UPS] and
 * dL_dsp [NSP][NS] (the system parameters) out; the gradient of the discrete
 * map with the recorded step sequence frozen. Systems whose step count
 * exceeded the tape get MPGOS_INSTANCE_TAPE_OVERFLOW and no gradient.
 * Asynchronous on the solver's stream. */
int mpgos_cb_solve_record(mpgos_cb_solver* solver, int32_t max_steps, int32_t segment);
int mpgos_cb_adjoint(mpgos_cb_solver* solver, const double* dL_dxT, double* dL_dx0, double* dL_dsp);
int mpgos_cb_tape_info(const mpgos_cb_solver* solver, mpgos_pt_tape* tape);

/* Coupled kernel table of a coupled-system plugin, or NULL. */
typedef const mpgos_cb_kernels* (*mpgos_cb_system_fn)(int32_t algorithm, int32_t precision_bytes);
const mpgos_cb_kernels* mpgos_cb_system_kernels(int32_t algorithm, int32_t precision_bytes);

/* ---- entry point exported by every system plugin --------------------- */
/* Kernel table for (algorithm, precision_bytes), or NULL if not compiled. */
typedef const mpgos_pt_kernels* (*mpgos_pt_system_fn)(int32_t algorithm, int32_t precision_bytes);
const mpgos_pt_kernels* mpgos_pt_system_kernels(int32_t algorithm, int32_t precision_bytes);

#ifdef __cplusplus
}
#endif

#endif /* MPGOS_H */
