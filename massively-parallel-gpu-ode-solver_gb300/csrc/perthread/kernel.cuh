// Per-thread ensemble solver kernels for sm_103a.
//
// One ODE instance per lane, the whole integration loop of one launch inside
// the kernel, state in registers, SoA [field][NT] arrays in HBM - the execution
// model of the reference kernel SingleSystem_PerThread
// (SourceCodes/SingleSystem_PerThread_Solver.cuh:11-437), re-organised for GB300:
//
//  * The per-instance loop is a state machine that performs one step attempt
//    per iteration. A lane whose instance has finished writes it back and, in
//    PERSISTENT mode, pulls the next instance index from a device work counter
//    inside the same iteration, so the warp keeps stepping with all lanes busy
//    instead of idling until its slowest lane finishes. This replaces the
//    reference's one-thread-one-instance launch and its NumberOfActiveThreads
//    tail guard (SingleSystem_PerThread_Solver.cuh:91).
//  * Tolerances, event options and the shared parameters are staged once per
//    CTA in shared memory behind a barrier.
//  * Every instance loop is bounded by MaximumAttempts; an instance that hits
//    it stops with MPGOS_INSTANCE_ATTEMPT_LIMIT instead of spinning.
//  * Per-instance status flags and accepted/rejected step counts replace the
//    reference's device printf warnings.
//
// The user hooks (PerThread_OdeFunction, PerThread_EventFunction,
// PerThread_ActionAfterEventDetection, PerThread_ActionAfterSuccessfulTimeStep,
// PerThread_Initialization, PerThread_Finalization) must be declared before
// this header is included, exactly as with the reference interface header.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "numerics.cuh"

// Largest block the kernels are compiled for (register budget 65536 / 256).
#ifndef MPGOS_MAX_BLOCK
#define MPGOS_MAX_BLOCK 256
#endif

namespace mpgos {
namespace pt {

template <int SD_, int NCP_, int NSP_, int NISP_, int NE_, int NA_, int NIA_>
struct Shape {
    static constexpr int SD = SD_, NCP = NCP_, NSP = NSP_, NISP = NISP_, NE = NE_, NA = NA_, NIA = NIA_;
};

// Kernel arguments in the kernel's precision (the reference passes the same
// information as Struct_ThreadConfiguration / Struct_GlobalVariables /
// Struct_SharedMemoryUsage / Struct_SolverOptions,
// SingleSystem_PerThread_Interface.cuh:72-115).
template <class P>
struct Args {
    long long nt;
    long long n_active;
    P* td;
    P* x;
    P* t;
    P* cp;
    const P* sp;
    const int* spi;
    P* acc;
    int* acci;
    const P* rtol;
    const P* atol;
    const P* etol;
    const int* edir;
    int* didx;
    P* dtime;
    P* dstate;
    int* status;
    int* n_acc;
    int* n_rej;
    unsigned int* work;
    const int* order;  // instance of each work item (MPGOS_WORK_ORDER), or null: the identity
    int prefer_shared;
    Options<P> o;
    Tape tape;
};

// Instance integrated for work item k (the static mapping's lane / stride
// index or the persistent queue's count): the runtime's order, or k itself.
template <class P>
__device__ __forceinline__ long long instance_at(const Args<P>& a, long long k)
{
    return a.order != nullptr ? static_cast<long long>(a.order[k]) : k;
}

// Registers of one instance between step attempts.
template <class S, class P>
struct Instance {
    static constexpr int SD = S::SD;
    long long i;
    P td[2];
    P x[SD];
    P cp[AtLeastOne<S::NCP>::value];
    P acc[AtLeastOne<S::NA>::value];
    int acci[AtLeastOne<S::NIA>::value];
    P ga[AtLeastOne<S::NE>::value];
    P t, dt, new_dt, dense_next;
    int didx, skipped, terminate, udt, status, nacc, nrej;
    long long attempts;
};

// Block-shared copies of the per-block constant data.
template <class S, class P>
struct Staged {
    P* sp;
    int* spi;
    const P* rtol;
    const P* atol;
    const P* etol;
    const int* edir;
    const float* lrtol;  // log2 of the tolerances (FAST_CONTROL)
    const float* latol;
};

template <class S, int ALG, class P, int MODE>
struct Solver {
    static constexpr int SD = S::SD, NCP = S::NCP, NSP = S::NSP, NISP = S::NISP;
    static constexpr int NE = S::NE, NA = S::NA, NIA = S::NIA;
    static constexpr bool PERSISTENT = (MODE & MPGOS_MODE_PERSISTENT) != 0;
    // FAST_CONTROL and FP32_STAGE apply to FP64 instances of the adaptive scheme.
    static constexpr bool IS_DOUBLE = sizeof(P) == 8;
    static constexpr bool FAST = ((MODE & MPGOS_MODE_FAST_CONTROL) != 0) && IS_DOUBLE && ALG == MPGOS_RKCK45;
    static constexpr bool F32S = ((MODE & MPGOS_MODE_FP32_STAGE) != 0) && IS_DOUBLE && ALG == MPGOS_RKCK45;
    static constexpr bool RECORD = ((MODE & MODE_RECORD) != 0) && IS_DOUBLE;
    using Inst = Instance<S, P>;

    // Load instance i and run the start-of-launch part of the reference loop
    // (SingleSystem_PerThread_Solver.cuh:117-193).
    __device__ static void begin(Inst& s, long long i, const Args<P>& a, const Staged<S, P>& g,
                                 float* cpf, float* accf)
    {
        const long long nt = a.nt;
        s.i = i;
#pragma unroll
        for (int k = 0; k < 2; k++) s.td[k] = a.td[i + k * nt];
#pragma unroll
        for (int k = 0; k < SD; k++) s.x[k] = a.x[i + k * nt];
#pragma unroll
        for (int k = 0; k < NCP; k++) s.cp[k] = a.cp[i + k * nt];
#pragma unroll
        for (int k = 0; k < NA; k++) s.acc[k] = a.acc[i + k * nt];
#pragma unroll
        for (int k = 0; k < NIA; k++) s.acci[k] = a.acci[i + k * nt];
        s.t          = a.t[i];
        s.dt         = a.o.initial_dt;
        s.new_dt     = a.o.initial_dt;
        s.didx       = a.didx[i];
        s.skipped    = 0;
        s.terminate  = 0;
        s.udt        = 0;
        s.status     = 0;
        s.nacc       = 0;
        s.nrej       = 0;
        s.attempts   = 0;
        s.dense_next = s.t;

        const int ti = static_cast<int>(i), nti = static_cast<int>(nt);
        PerThread_Initialization(ti, nti, s.didx, s.t, s.dt, s.td, s.x, s.cp, g.sp, g.spi, s.acc, s.acci);
        if (NE > 0)
            PerThread_EventFunction(ti, nti, s.ga, s.t, s.dt, s.td, s.x, s.cp, g.sp, g.spi, s.acc, s.acci);
        if (a.o.ndo > 0)
            dense_store<SD, P>(i, nt, 1, s.didx, a.o.ndo, a.dtime, a.dstate, s.t, s.x, s.skipped,
                               s.dense_next, a.o.dense_min_dt, s.td[1]);
        if (F32S) refresh_f32(s, cpf, accf);
        if constexpr (RECORD) {
            // checkpoint 0: the state the first step starts from
            a.tape.ckpt_t[i] = s.t;
#pragma unroll
            for (int d = 0; d < SD; d++) a.tape.ckpt_x[d * nt + i] = s.x[d];
        }
    }

    __device__ static void refresh_f32(const Inst& s, float* cpf, float* accf)
    {
#pragma unroll
        for (int k = 0; k < NCP; k++) cpf[k] = static_cast<float>(s.cp[k]);
#pragma unroll
        for (int k = 0; k < NA; k++) accf[k] = static_cast<float>(s.acc[k]);
    }

    // One step attempt: the body of the reference's while loop
    // (SingleSystem_PerThread_Solver.cuh:197-393).
    __device__ static void attempt(Inst& s, const Args<P>& a, const Staged<S, P>& g, float* cpf,
                                   float* spf, float* accf)
    {
        const Options<P>& o = a.o;
        if (s.attempts >= o.max_attempts) {
            s.status |= MPGOS_INSTANCE_ATTEMPT_LIMIT;
            s.terminate = 1;
            return;
        }
        s.attempts++;

        const int ti = static_cast<int>(s.i), nti = static_cast<int>(a.nt);
        int update = 1, finite = 1, end_reached = 0;
        P xn[SD];
        P err[SD];
        s.dt = s.new_dt;
        {
            // Clamp to the end of the time domain. FAST_CONTROL compares the
            // positive step with the remaining interval as int64 bit patterns
            // (exact, also when the remainder is negative) instead of in FP64.
            const P rem = s.td[1] - s.t;
            bool clamp;
            if constexpr (FAST) clamp = bits_of(s.dt) > bits_of(rem);
            else clamp = s.dt > rem;
            if (clamp) {
                s.dt        = rem;
                end_reached = 1;
            }
        }

        if (ALG == MPGOS_RK4) {
            step_rk4<SD, P>(ti, nti, s.t, s.dt, s.x, xn, finite, s.cp, g.sp, g.spi, s.acc, s.acci);
            control_rk4<P>(o, finite, s.terminate, s.new_dt, s.status);
        } else {
            if constexpr (F32S) {
                step_rkck45_f32stage<SD, NCP, NA>(ti, nti, s.t, s.dt, s.x, xn, err, finite, cpf, spf, g.spi,
                                                  accf, s.acci);
            } else {
                step_rkck45<SD, P, FAST>(ti, nti, s.t, s.dt, s.x, xn, err, finite, s.cp, g.sp, g.spi, s.acc,
                                         s.acci);
            }
            if constexpr (FAST) {
                control_rkck45_fast<SD>(o, s.dt, s.x, xn, err, g.rtol, g.atol, g.lrtol, g.latol, update, finite,
                                        s.terminate, s.new_dt, s.status);
            } else {
                control_rkck45_plain<SD, P>(o, s.dt, s.x, xn, err, g.rtol, g.atol, update, finite, s.terminate,
                                            s.new_dt, s.status);
            }
        }

        P gn[AtLeastOne<NE>::value];
        if (NE > 0) {
            PerThread_EventFunction(ti, nti, gn, s.t + s.dt, s.dt, s.td, xn, s.cp, g.sp, g.spi, s.acc, s.acci);
            event_step_control<NE, P>(update, s.terminate, s.ga, gn, g.etol, g.edir, s.dt, s.new_dt, o.min_dt,
                                      s.status);
        }

        if (update == 1) {
            s.nacc++;
            s.t += s.dt;
#pragma unroll
            for (int k = 0; k < SD; k++) s.x[k] = xn[k];

            PerThread_ActionAfterSuccessfulTimeStep(ti, nti, s.udt, s.t, s.dt, s.td, s.x, s.cp, g.sp, g.spi,
                                                    s.acc, s.acci);
            if (NE > 0) {
                for (int e = 0; e < NE; e++) {
                    if (event_detected<P>(s.ga[e], gn[e], g.etol[e], g.edir[e]))
                        PerThread_ActionAfterEventDetection(ti, nti, e, s.udt, s.t, s.dt, s.td, s.x, s.cp, g.sp,
                                                            g.spi, s.acc, s.acci);
                }
                PerThread_EventFunction(ti, nti, gn, s.t, s.dt, s.td, s.x, s.cp, g.sp, g.spi, s.acc, s.acci);
#pragma unroll
                for (int e = 0; e < NE; e++) s.ga[e] = gn[e];
            }
            if (o.ndo > 0) {
                const int store = dense_condition<P>(s.t, s.dense_next, s.didx, s.skipped, end_reached, s.udt,
                                                     o.ndo, o.dense_freq);
                dense_store<SD, P>(s.i, a.nt, store, s.didx, o.ndo, a.dtime, a.dstate, s.t, s.x, s.skipped,
                                   s.dense_next, o.dense_min_dt, s.td[1]);
            }
            if (F32S && NA > 0) refresh_f32(s, cpf, accf);
            if constexpr (RECORD) {
                // frozen step size of accepted step nacc, checkpoint every seg steps
                const int k = s.nacc - 1;
                if (k < a.tape.max_steps) {
                    a.tape.dt[static_cast<long long>(k) * a.nt + s.i] = s.dt;
                    if (s.nacc % a.tape.seg == 0) {
                        const long long c = s.nacc / a.tape.seg;
                        a.tape.ckpt_t[c * a.nt + s.i] = s.t;
#pragma unroll
                        for (int d = 0; d < SD; d++) a.tape.ckpt_x[(c * SD + d) * a.nt + s.i] = s.x[d];
                    }
                } else {
                    s.status |= MPGOS_INSTANCE_TAPE_OVERFLOW;
                }
            }
            if ((end_reached == 1) || (s.udt == 1)) s.terminate = 1;
        } else {
            s.nrej++;
        }
    }

    // Finalization hook and write-back (SingleSystem_PerThread_Solver.cuh:397-435).
    __device__ static void end(Inst& s, const Args<P>& a, const Staged<S, P>& g)
    {
        const long long i = s.i, nt = a.nt;
        const int ti = static_cast<int>(i), nti = static_cast<int>(nt);
        PerThread_Finalization(ti, nti, s.didx, s.t, s.dt, s.td, s.x, s.cp, g.sp, g.spi, s.acc, s.acci);
#pragma unroll
        for (int k = 0; k < 2; k++) a.td[i + k * nt] = s.td[k];
#pragma unroll
        for (int k = 0; k < SD; k++) a.x[i + k * nt] = s.x[k];
#pragma unroll
        for (int k = 0; k < NCP; k++) a.cp[i + k * nt] = s.cp[k];
#pragma unroll
        for (int k = 0; k < NA; k++) a.acc[i + k * nt] = s.acc[k];
#pragma unroll
        for (int k = 0; k < NIA; k++) a.acci[i + k * nt] = s.acci[k];
        a.t[i]    = s.t;
        a.didx[i] = s.didx;
        if (a.status) a.status[i] = s.status;
        if (a.n_acc) a.n_acc[i] = s.nacc;
        if (a.n_rej) a.n_rej[i] = s.nrej;
        if constexpr (RECORD) a.tape.n_steps[i] = s.nacc;
    }

    // Next instance for a lane whose instance finished. Static mapping: the
    // grid stride (a grid smaller than the ensemble gives every lane several
    // instances in sequence, MPGOS_INSTANCES_PER_THREAD; with one lane per
    // instance the stride ends the lane). Persistent: warp-aggregated atomic
    // on the work counter, which counts instances handed out beyond the first
    // one per lane.
    __device__ static long long next_index(const Args<P>& a, long long total_threads, long long current)
    {
        if (!PERSISTENT) return current + total_threads;
        const unsigned mask   = __activemask();
        const int lane        = threadIdx.x & 31;
        const int leader      = __ffs(mask) - 1;
        const unsigned rank   = __popc(mask & ((1u << lane) - 1u));
        unsigned base = 0;
        if (lane == leader) base = atomicAdd(a.work, static_cast<unsigned>(__popc(mask)));
        base = __shfl_sync(mask, base, leader);
        return total_threads + static_cast<long long>(base) + rank;
    }
};

// Dynamic shared memory: [NSP] P, then [NISP] int.
template <class S, class P>
__host__ __device__ constexpr size_t dynamic_smem_bytes()
{
    return sizeof(P) * S::NSP + sizeof(int) * S::NISP;
}

template <class S, int ALG, class P, int MODE>
__global__ void __launch_bounds__(MPGOS_MAX_BLOCK) perthread_kernel(Args<P> a)
{
    using Sv = Solver<S, ALG, P, MODE>;
    constexpr int SD = S::SD, NSP = S::NSP, NISP = S::NISP, NE = S::NE;
    constexpr bool ADAPTIVE = (ALG == MPGOS_RKCK45);

    extern __shared__ __align__(16) unsigned char mpgos_dyn_smem[];
    __shared__ P s_rtol[ADAPTIVE ? SD : 1];
    __shared__ P s_atol[ADAPTIVE ? SD : 1];
    __shared__ P s_etol[AtLeastOne<NE>::value];
    __shared__ int s_edir[AtLeastOne<NE>::value];
    __shared__ float s_spf[AtLeastOne<NSP>::value];
    __shared__ float s_lrtol[ADAPTIVE ? SD : 1];
    __shared__ float s_latol[ADAPTIVE ? SD : 1];

    P* dyn_sp   = reinterpret_cast<P*>(mpgos_dyn_smem);
    int* dyn_spi = reinterpret_cast<int*>(mpgos_dyn_smem + sizeof(P) * NSP);

    for (int k = threadIdx.x; k < SD; k += blockDim.x) {
        if (ADAPTIVE) {
            s_rtol[k] = a.rtol[k];
            s_atol[k] = a.atol[k];
            if constexpr (Sv::FAST) {
                s_lrtol[k] = log2_nonneg(a.rtol[k]);
                s_latol[k] = log2_nonneg(a.atol[k]);
            }
        }
    }
    for (int k = threadIdx.x; k < NE; k += blockDim.x) {
        s_etol[k] = a.etol[k];
        s_edir[k] = a.edir[k];
    }
    if (a.prefer_shared) {
        for (int k = threadIdx.x; k < NSP; k += blockDim.x) dyn_sp[k] = a.sp[k];
        for (int k = threadIdx.x; k < NISP; k += blockDim.x) dyn_spi[k] = a.spi[k];
    }
    if (Sv::F32S) {
        for (int k = threadIdx.x; k < NSP; k += blockDim.x) s_spf[k] = static_cast<float>(a.sp[k]);
    }
    __syncthreads();

    Staged<S, P> g;
    g.sp   = a.prefer_shared ? dyn_sp : const_cast<P*>(a.sp);
    g.spi  = a.prefer_shared ? dyn_spi : const_cast<int*>(a.spi);
    g.rtol = s_rtol;
    g.atol = s_atol;
    g.etol = s_etol;
    g.edir = s_edir;
    g.lrtol = s_lrtol;
    g.latol = s_latol;

    float cpf[AtLeastOne<S::NCP>::value];
    float accf[AtLeastOne<S::NA>::value];

    const long long total = static_cast<long long>(gridDim.x) * blockDim.x;
    long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if constexpr ((MODE & MODE_RECONVERGE) != 0) {
        // Lanes of this warp that integrate; every iteration ends with a
        // ballot over them, which reconverges the warp once per step attempt
        // (divergent accept/reject, event and end-of-instance paths can
        // otherwise leave lanes running the next attempt's stages in
        // separate groups).
        unsigned live = __ballot_sync(__activemask(), i < a.n_active);
        if (i >= a.n_active) return;
        typename Sv::Inst s;
        Sv::begin(s, instance_at(a, i), a, g, cpf, accf);
        while (true) {
            bool stop = false;
            if (s.terminate) {
                Sv::end(s, a, g);
                i = Sv::next_index(a, total, i);
                if (i >= a.n_active) stop = true;
                else Sv::begin(s, instance_at(a, i), a, g, cpf, accf);
            }
            if (!stop) Sv::attempt(s, a, g, cpf, s_spf, accf);
            live = __ballot_sync(live, !stop);
            if (stop) break;
        }
    } else {
        if (i >= a.n_active) return;
        typename Sv::Inst s;
        Sv::begin(s, instance_at(a, i), a, g, cpf, accf);
        while (true) {
            if (s.terminate) {
                Sv::end(s, a, g);
                i = Sv::next_index(a, total, i);
                if (i >= a.n_active) break;
                Sv::begin(s, instance_at(a, i), a, g, cpf, accf);
            }
            Sv::attempt(s, a, g, cpf, s_spf, accf);
        }
    }
}

}  // namespace pt
}  // namespace mpgos

#include "df_solver.cuh"
#include "split_solver.cuh"

namespace mpgos {
namespace pt {

// ---------------------------------------------------------------------------
// Kernel table: the launch side of the plugin ABI (mpgos_pt_kernels in mpgos.h).
// ---------------------------------------------------------------------------
template <class P>
Args<P> make_args(const mpgos_pt_launch& L)
{
    Args<P> a;
    a.nt            = L.nt;
    a.n_active      = L.n_active;
    a.td            = static_cast<P*>(L.time_domain);
    a.x             = static_cast<P*>(L.actual_state);
    a.t             = static_cast<P*>(L.actual_time);
    a.cp            = static_cast<P*>(L.control_parameters);
    a.sp            = static_cast<const P*>(L.shared_parameters);
    a.spi           = L.integer_shared_parameters;
    a.acc           = static_cast<P*>(L.accessories);
    a.acci          = L.integer_accessories;
    a.rtol          = static_cast<const P*>(L.relative_tolerance);
    a.atol          = static_cast<const P*>(L.absolute_tolerance);
    a.etol          = static_cast<const P*>(L.event_tolerance);
    a.edir          = L.event_direction;
    a.didx          = L.dense_index;
    a.dtime         = static_cast<P*>(L.dense_time);
    a.dstate        = static_cast<P*>(L.dense_state);
    a.status        = L.status;
    a.n_acc         = L.accepted_steps;
    a.n_rej         = L.rejected_steps;
    a.work          = L.work_counter;
    a.order         = L.instance_order;
    a.prefer_shared = L.prefer_shared;
    a.o.initial_dt   = static_cast<P>(L.initial_dt);
    a.o.max_dt       = static_cast<P>(L.max_dt);
    a.o.min_dt       = static_cast<P>(L.min_dt);
    a.o.grow         = static_cast<P>(L.grow_limit);
    a.o.shrink       = static_cast<P>(L.shrink_limit);
    a.o.dense_min_dt = static_cast<P>(L.dense_min_dt);
    a.o.min_dt_guard = a.o.min_dt * static_cast<P>(1.01);
    a.o.dense_freq   = L.dense_save_frequency;
    a.o.ndo          = L.ndo;
    a.o.max_attempts = L.max_attempts;
    return a;
}

// Adjoint launchers, filled in by adjoint.cuh's AdjointTable where compiled.
using RecordFn  = int (*)(const mpgos_pt_launch*, const mpgos_pt_tape*, int, int, size_t, void*);
using AdjointFn = int (*)(const mpgos_pt_launch*, const mpgos_pt_tape*, const double*, double*, double*, int, int,
                          size_t, void*);

}  // namespace pt
}  // namespace mpgos

#include "dense_interp.cuh"

namespace mpgos {
namespace pt {

// The double-float kernels of one scheme and arithmetic (ARITH: DF_STAGE or
// SPLIT) with their twins: persistent mapping (MPGOS_MODE_PERSISTENT), warp
// reconvergence (MODE_RECONVERGE), out-of-line right-hand side
// (MODE_OUTLINE_RHS) and the adjoint's recording pass (MODE_RECORD, static or
// persistent). get() takes the mode without the ARITH bit.
template <class S, int ALG, int ARITH>
struct DfKernelSet {
    template <int M>
    static void* k()
    {
        if constexpr (ARITH == MPGOS_MODE_DF_STAGE)
            return reinterpret_cast<void*>(&perthread_df_kernel<S, M | MPGOS_MODE_DF_STAGE, ALG>);
        else
            return reinterpret_cast<void*>(&perthread_split_kernel<S, M | MPGOS_MODE_SPLIT, ALG>);
    }

    static void* get(int mode)
    {
        constexpr int PS = MPGOS_MODE_PERSISTENT, R = MODE_RECONVERGE, O = MODE_OUTLINE_RHS, REC = MODE_RECORD;
        switch (mode) {
            case 0: return k<0>();
            case PS: return k<PS>();
            case R: return k<R>();
            case R | PS: return k<R | PS>();
            case O: return k<O>();
            case O | PS: return k<O | PS>();
            case O | R: return k<O | R>();
            case O | R | PS: return k<O | R | PS>();
            case REC: return k<REC>();
            case REC | PS: return k<REC | PS>();
            default: return nullptr;
        }
    }
};

#ifdef MPGOS_PLUGIN_PARTS
// A system plugin built from several translation units compiles each
// double-float kernel set in a unit of its own, in parallel; this dispatcher
// (defined by the plugin's main unit, plugin_export.cuh) returns them.
void* plugin_part_kernel(int arith, int alg, int mode);
#endif

template <class S, int ALG>
void* double_float_kernel(int arith, int mode)
{
#ifdef MPGOS_PLUGIN_PARTS
    return plugin_part_kernel(arith, ALG, mode);
#else
    return arith == MPGOS_MODE_DF_STAGE ? DfKernelSet<S, ALG, MPGOS_MODE_DF_STAGE>::get(mode)
                                        : DfKernelSet<S, ALG, MPGOS_MODE_SPLIT>::get(mode);
#endif
}

template <class S, int ALG, class P>
struct KernelTable {
    static constexpr bool DOUBLE_ADAPTIVE = sizeof(P) == 8 && ALG == MPGOS_RKCK45;
    static constexpr bool DOUBLE = sizeof(P) == 8;  // DF_STAGE and SPLIT: both schemes
    static constexpr int MODES = MPGOS_MODE_PERSISTENT |
                                 (DOUBLE_ADAPTIVE ? (MPGOS_MODE_FAST_CONTROL | MPGOS_MODE_FP32_STAGE) : 0) |
                                 (DOUBLE ? (MPGOS_MODE_DF_STAGE | MPGOS_MODE_SPLIT) : 0);

    // Modes a table can run; the runtime only asks for these. MODE_RECONVERGE
    // selects the twin of each kernel with the per-attempt warp ballot,
    // MODE_OUTLINE_RHS (double-float kernels only) the twin with the
    // right-hand side out of line.
    static void* kernel_for(int mode)
    {
        if constexpr (DOUBLE) {
            for (int arith : {MPGOS_MODE_DF_STAGE, MPGOS_MODE_SPLIT})
                if (mode & arith) return double_float_kernel<S, ALG>(arith, mode & ~arith);
        }
        if (mode & MODE_OUTLINE_RHS) return nullptr;
        const int R = mode & MODE_RECONVERGE;
        mode &= ~MODE_RECONVERGE;
        switch (mode) {
            case 0: return R ? fp<MODE_RECONVERGE>() : fp<0>();
            case 2: return R ? fp<MODE_RECONVERGE | 2>() : fp<2>();
            default: break;
        }
        if constexpr (DOUBLE_ADAPTIVE) {
            switch (mode) {
                case 1: return R ? fp<MODE_RECONVERGE | 1>() : fp<1>();
                case 3: return R ? fp<MODE_RECONVERGE | 3>() : fp<3>();
                case 5: return R ? fp<MODE_RECONVERGE | 5>() : fp<5>();
                case 7: return R ? fp<MODE_RECONVERGE | 7>() : fp<7>();
                default: break;
            }
        }
        return nullptr;
    }

    template <int M>
    static void* fp()
    {
        return reinterpret_cast<void*>(&perthread_kernel<S, ALG, P, M>);
    }

    static int launch(const mpgos_pt_launch* L, int grid, int block, size_t smem, void* stream)
    {
        void* fn = kernel_for(L->mode);
        if (fn == nullptr) return static_cast<int>(cudaErrorInvalidValue);
        Args<P> a = make_args<P>(*L);
        void* params[] = {&a};
        return static_cast<int>(cudaLaunchKernel(fn, dim3(grid), dim3(block), params, smem,
                                                 static_cast<cudaStream_t>(stream)));
    }

    static int occupancy(int32_t mode, int block, size_t smem, int* blocks)
    {
        void* fn = kernel_for(mode);
        if (fn == nullptr) return static_cast<int>(cudaErrorInvalidValue);
        return static_cast<int>(cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, fn, block, smem));
    }

    static const mpgos_pt_kernels* get(const char* name, RecordFn record = nullptr, AdjointFn adjoint = nullptr)
    {
        static mpgos_pt_kernels table = {
            MPGOS_ABI_VERSION,
            {S::SD, S::NCP, S::NSP, S::NISP, S::NE, S::NA, S::NIA, ALG, static_cast<int32_t>(sizeof(P)), MODES},
            name,
            &launch,
            &occupancy,
            record,
            adjoint,
            &DenseInterpTable<S, P>::launch};
        return &table;
    }
};

}  // namespace pt
}  // namespace mpgos
