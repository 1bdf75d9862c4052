// Host runtime of the GB300 ensemble solver: implementation of the C-ABI in
// mpgos.h (libmpgos_runtime.so).
//
// It plays the role of the reference's host object ProblemSolver
// (SourceCodes/SingleSystem_PerThread_Interface.cuh:117-208, :309-1312):
// pinned host + device SoA buffers, one stream and one event per solver,
// option handling, host<->device synchronisation and the kernel launch. The
// kernels themselves come from a system plugin through mpgos_pt_kernels.
// Beyond the reference it adds CUDA-graph capture of multi-phase runs, CUDA
// event timing, per-instance status/step statistics and an autotuner.
#include "mpgos.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#define MPGOS_EXPORT extern "C" __attribute__((visibility("default")))

namespace {

thread_local std::string g_last_error;

int fail(int code, const char* fmt, ...)
{
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

#define MPGOS_CUDA(call)                                                                          \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess)                                                                    \
            return fail(MPGOS_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_),   \
                        __FILE__, __LINE__);                                                      \
    } while (0)

constexpr int kVarCount = 64;

// Device address of the static tape array on `device` (defined with the
// array, near mpgos_pt_solve_record_static).
int static_tape_base(int device, unsigned char** base);

// Host and device copy of one SoA array.
struct Buffer {
    void* host   = nullptr;
    void* device = nullptr;
    int64_t count = 0;   // elements
    size_t elem   = 0;   // bytes per element
    size_t bytes() const { return static_cast<size_t>(count) * elem; }
};

struct GraphKey {
    int32_t n_phases;
    int32_t stream_accessory;
    void* phase_output;
    uint64_t generation;
    bool operator<(const GraphKey& o) const
    {
        return std::tie(n_phases, stream_accessory, phase_output, generation) <
               std::tie(o.n_phases, o.stream_accessory, o.phase_output, o.generation);
    }
};

}  // namespace

// Entry for the coupled-solver runtime (runtime_coupled.cpp): same error slot.
namespace mpgos_runtime {
int set_error(int code, const char* msg)
{
    g_last_error = msg;
    return code;
}
}  // namespace mpgos_runtime

// work_order.cu: the longest-first instance order of MPGOS_WORK_ORDER
int mpgos_internal_order_instances(cudaStream_t stream, const int32_t* nacc, const int32_t* nrej, long long n,
                                   unsigned* scratch, int32_t* order, int sm_count);
int mpgos_internal_order_scratch_counters();

struct mpgos_pt_solver {
    const mpgos_pt_kernels* k = nullptr;
    mpgos_pt_shape shape{};
    int64_t nt  = 0;
    int32_t ndo = 0;
    int device  = 0;
    int sm_count = 0;
    std::string gpu_name;
    cudaStream_t stream = nullptr;
    cudaEvent_t sync_event = nullptr;
    cudaEvent_t timer_begin = nullptr, timer_end = nullptr;

    Buffer var[kVarCount];
    // device-only option arrays
    void* d_rtol = nullptr;
    void* d_atol = nullptr;
    void* d_etol = nullptr;
    int32_t* d_edir = nullptr;
    uint32_t* d_work = nullptr;
    std::vector<double> rtol, atol, etol;
    std::vector<int32_t> edir;

    // options (reference defaults, SingleSystem_PerThread_Interface.cuh:475-496)
    int block = 32;
    int64_t n_active = 0;
    double initial_dt = 1e-2, max_dt = 1e6, min_dt = 1e-12, grow = 5.0, shrink = 0.1, dense_min_dt = 0.0;
    int32_t dense_freq = 1;
    int32_t prefer_shared = 1;
    int32_t ipt = 1;  // instances per thread of the static mapping
    int32_t reconverge = -1;  // MPGOS_WARP_RECONVERGE; -1: by the system (events: 1)
    int32_t outline = 0;      // MPGOS_OUTLINE_RHS (double-float kernels)
    int32_t work_order = 0;   // MPGOS_WORK_ORDER
    int32_t* d_order = nullptr;           // [NT] instance of each work item
    unsigned* d_order_scratch = nullptr;  // counting-sort buckets
    int32_t mode = MPGOS_MODE_PLAIN;
    int64_t max_attempts = 10000000;
    uint64_t generation = 1;  // bumped by every change that alters a launch

    std::map<GraphKey, cudaGraphExec_t> graphs;
    std::vector<void*> checkpoint;  // device copies, one per checkpointed variable

    // adjoint tape (device memory, allocated by the first recording solve)
    mpgos_pt_tape tape{};
    size_t tape_bytes = 0;
    // Tape views into the static device scratch of mpgos_pt_solve_record_static;
    // use_static_tape selects which tape the reverse pass reads.
    mpgos_pt_tape static_tape{};
    bool use_static_tape = false;
};

namespace {

size_t prec(const mpgos_pt_solver* s) { return static_cast<size_t>(s->shape.precision_bytes); }

bool is_reference_variable(int32_t v) { return v >= MPGOS_TIME_DOMAIN && v <= MPGOS_DENSE_STATE && v != MPGOS_DENSE_OUTPUT; }
bool is_extension_variable(int32_t v) { return v >= MPGOS_STATUS && v <= MPGOS_REJECTED_STEPS; }

int check_solver(const mpgos_pt_solver* s)
{
    if (s == nullptr) return fail(MPGOS_ERR_ARGUMENT, "null solver handle");
    return MPGOS_OK;
}

// Upload a scalar option array (tolerances, event options) right away, as
// SolverOption does in the reference (SingleSystem_PerThread_Interface.cuh:679-694).
int push_option_arrays(mpgos_pt_solver* s)
{
    const size_t p = prec(s);
    auto put = [&](void* dst, const std::vector<double>& v) -> int {
        if (v.empty()) return MPGOS_OK;
        std::vector<unsigned char> tmp(v.size() * p);
        for (size_t i = 0; i < v.size(); i++) {
            if (p == 8) {
                double d = v[i];
                std::memcpy(&tmp[i * p], &d, p);
            } else {
                float f = static_cast<float>(v[i]);
                std::memcpy(&tmp[i * p], &f, p);
            }
        }
        MPGOS_CUDA(cudaMemcpy(dst, tmp.data(), tmp.size(), cudaMemcpyHostToDevice));
        return MPGOS_OK;
    };
    MPGOS_CUDA(cudaSetDevice(s->device));
    MPGOS_CUDA(cudaStreamSynchronize(s->stream));
    int rc;
    if ((rc = put(s->d_rtol, s->rtol)) != MPGOS_OK) return rc;
    if ((rc = put(s->d_atol, s->atol)) != MPGOS_OK) return rc;
    if ((rc = put(s->d_etol, s->etol)) != MPGOS_OK) return rc;
    if (!s->edir.empty())
        MPGOS_CUDA(cudaMemcpy(s->d_edir, s->edir.data(), s->edir.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    return MPGOS_OK;
}

void fill_launch(const mpgos_pt_solver* s, mpgos_pt_launch& L, int32_t mode)
{
    std::memset(&L, 0, sizeof(L));
    L.nt                   = s->nt;
    L.n_active             = s->n_active;
    L.ndo                  = s->ndo;
    L.mode                 = mode;
    L.prefer_shared        = s->prefer_shared;
    L.dense_save_frequency = s->dense_freq;
    L.max_attempts         = s->max_attempts;
    L.initial_dt           = s->initial_dt;
    L.max_dt               = s->max_dt;
    L.min_dt               = s->min_dt;
    L.grow_limit           = s->grow;
    L.shrink_limit         = s->shrink;
    L.dense_min_dt         = s->dense_min_dt;
    L.time_domain               = s->var[MPGOS_TIME_DOMAIN].device;
    L.actual_state              = s->var[MPGOS_ACTUAL_STATE].device;
    L.actual_time               = s->var[MPGOS_ACTUAL_TIME].device;
    L.control_parameters        = s->var[MPGOS_CONTROL_PARAMETERS].device;
    L.shared_parameters         = s->var[MPGOS_SHARED_PARAMETERS].device;
    L.integer_shared_parameters = static_cast<const int32_t*>(s->var[MPGOS_INTEGER_SHARED_PARAMETERS].device);
    L.accessories               = s->var[MPGOS_ACCESSORIES].device;
    L.integer_accessories       = static_cast<int32_t*>(s->var[MPGOS_INTEGER_ACCESSORIES].device);
    L.relative_tolerance        = s->d_rtol;
    L.absolute_tolerance        = s->d_atol;
    L.event_tolerance           = s->d_etol;
    L.event_direction           = s->d_edir;
    L.dense_index               = static_cast<int32_t*>(s->var[MPGOS_DENSE_INDEX].device);
    L.dense_time                = s->var[MPGOS_DENSE_TIME].device;
    L.dense_state               = s->var[MPGOS_DENSE_STATE].device;
    L.status                    = static_cast<int32_t*>(s->var[MPGOS_STATUS].device);
    L.accepted_steps            = static_cast<int32_t*>(s->var[MPGOS_ACCEPTED_STEPS].device);
    L.rejected_steps            = static_cast<int32_t*>(s->var[MPGOS_REJECTED_STEPS].device);
    L.work_counter              = s->d_work;
}

size_t dynamic_smem(const mpgos_pt_solver* s)
{
    return prec(s) * static_cast<size_t>(s->shape.nsp) + sizeof(int32_t) * static_cast<size_t>(s->shape.nisp);
}

// Bit 32 of a launch mode selects the kernels with the per-attempt warp
// ballot (MPGOS_WARP_RECONVERGE; plugin side: MODE_RECONVERGE), bit 64 the
// double-float kernels with the right-hand side out of line
// (MPGOS_OUTLINE_RHS; plugin side: MODE_OUTLINE_RHS).
constexpr int32_t kModeReconverge = 32;
constexpr int32_t kModeOutlineRhs = 64;

int32_t effective_mode(const mpgos_pt_solver* s, int32_t mode)
{
    int32_t m = mode & (s->shape.modes | MPGOS_MODE_PERSISTENT);
    if (m & MPGOS_MODE_SPLIT) {
        m = MPGOS_MODE_SPLIT | (m & MPGOS_MODE_PERSISTENT);
        if (s->outline) m |= kModeOutlineRhs;
    } else if (m & MPGOS_MODE_DF_STAGE) {
        m = MPGOS_MODE_DF_STAGE | (m & MPGOS_MODE_PERSISTENT);
        if (s->outline) m |= kModeOutlineRhs;
    } else if (m & MPGOS_MODE_FP32_STAGE) {
        m |= MPGOS_MODE_FAST_CONTROL;  // compiled together
    }
    const bool rc = s->reconverge >= 0 ? s->reconverge != 0 : s->shape.ne > 0;
    return rc ? (m | kModeReconverge) : m;
}

int grid_for(const mpgos_pt_solver* s, int32_t mode, int block, int* grid)
{
    const int64_t blocks_needed = (s->n_active + block - 1) / block;
    int64_t g = blocks_needed;
    if (!(mode & MPGOS_MODE_PERSISTENT) && s->ipt > 1) {
        const int64_t per_block = static_cast<int64_t>(block) * s->ipt;
        g = (s->n_active + per_block - 1) / per_block;
    }
    if (mode & MPGOS_MODE_PERSISTENT) {
        int per_sm = 0;
        int rc = s->k->occupancy(mode, block, dynamic_smem(s), &per_sm);
        if (rc != 0) return fail(MPGOS_ERR_CUDA, "occupancy query failed: %s", cudaGetErrorString((cudaError_t)rc));
        if (per_sm < 1) per_sm = 1;
        g = std::min<int64_t>(blocks_needed, static_cast<int64_t>(per_sm) * s->sm_count);
    }
    if (g > 0x7FFFFFFF) return fail(MPGOS_ERR_ARGUMENT, "grid too large");
    *grid = static_cast<int>(std::max<int64_t>(g, 0));
    return MPGOS_OK;
}

// Enqueue one Solve() (work-counter reset + kernel) on the stream.
int enqueue_solve(mpgos_pt_solver* s, int32_t mode, int block)
{
    if (s->n_active <= 0) return MPGOS_OK;
    const int32_t m = effective_mode(s, mode);
    int grid = 0;
    int rc = grid_for(s, m, block, &grid);
    if (rc != MPGOS_OK) return rc;
    if (m & MPGOS_MODE_PERSISTENT) MPGOS_CUDA(cudaMemsetAsync(s->d_work, 0, sizeof(uint32_t), s->stream));
    mpgos_pt_launch L;
    fill_launch(s, L, m);
    if (s->work_order && s->d_order != nullptr) {
        // longest first by the attempts of the previous launch (on the stream,
        // so a graph of phases captures it with the launch)
        rc = mpgos_internal_order_instances(s->stream, L.accepted_steps, L.rejected_steps, s->n_active,
                                            s->d_order_scratch, s->d_order, s->sm_count);
        if (rc != 0) return fail(MPGOS_ERR_CUDA, "instance ordering failed: %s", cudaGetErrorString((cudaError_t)rc));
        L.instance_order = s->d_order;
    }
    rc = s->k->launch(&L, grid, block, dynamic_smem(s), s->stream);
    if (rc != 0) return fail(MPGOS_ERR_CUDA, "kernel launch failed: %s", cudaGetErrorString((cudaError_t)rc));
    return MPGOS_OK;
}

void clear_graphs(mpgos_pt_solver* s)
{
    for (auto& kv : s->graphs) cudaGraphExecDestroy(kv.second);
    s->graphs.clear();
}

std::string json_escape(const std::string& in)
{
    std::string out;
    for (char c : in) {
        if (c == '"' || c == '\\') out += '\\';
        out += c;
    }
    return out;
}

}  // namespace

// ===========================================================================
// C-ABI
// ===========================================================================

MPGOS_EXPORT const char* mpgos_last_error(void) { return g_last_error.c_str(); }
MPGOS_EXPORT int mpgos_abi_version(void) { return MPGOS_ABI_VERSION; }

MPGOS_EXPORT int mpgos_pt_create(const mpgos_pt_kernels* kernels, int64_t nt, int32_t ndo, int device,
                                 mpgos_pt_solver** out)
{
    g_last_error.clear();
    if (out == nullptr) return fail(MPGOS_ERR_ARGUMENT, "null output handle");
    *out = nullptr;
    if (kernels == nullptr) return fail(MPGOS_ERR_ARGUMENT, "null kernel table (system not compiled for this algorithm/precision?)");
    if (kernels->abi_version != MPGOS_ABI_VERSION)
        return fail(MPGOS_ERR_SHAPE, "kernel table ABI %d, runtime ABI %d", kernels->abi_version, MPGOS_ABI_VERSION);
    const mpgos_pt_shape& sh = kernels->shape;
    if (sh.sd < 1 || sh.ncp < 0 || sh.nsp < 0 || sh.nisp < 0 || sh.ne < 0 || sh.na < 0 || sh.nia < 0 ||
        (sh.precision_bytes != 4 && sh.precision_bytes != 8))
        return fail(MPGOS_ERR_SHAPE, "invalid kernel table shape");
    if (nt < 1 || nt > 0x7FFFFFFF) return fail(MPGOS_ERR_ARGUMENT, "number of instances %lld out of range 1..2^31-1", (long long)nt);
    if (ndo < 0) return fail(MPGOS_ERR_ARGUMENT, "negative number of dense-output points");

    mpgos_pt_solver* s = new mpgos_pt_solver();
    s->k = kernels;
    s->shape = sh;
    s->nt = nt;
    s->ndo = ndo;
    s->device = device;
    s->n_active = nt;

    auto cleanup = [&](int rc) {
        mpgos_pt_destroy(s);
        return rc;
    };
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return cleanup(fail(MPGOS_ERR_CUDA, "cudaSetDevice(%d): %s", device, cudaGetErrorString(e)));
    cudaDeviceProp prop;
    if ((e = cudaGetDeviceProperties(&prop, device)) != cudaSuccess)
        return cleanup(fail(MPGOS_ERR_CUDA, "cudaGetDeviceProperties: %s", cudaGetErrorString(e)));
    s->sm_count = prop.multiProcessorCount;
    s->gpu_name = prop.name;
    s->block = prop.warpSize;  // reference default: one warp (:343)
    {
        // the static tape of mpgos_pt_solve_record_static: its device module
        // is loaded (and its array reserved) here, at solver creation, not at
        // the first recording call
        unsigned char* base = nullptr;
        int rc0 = static_tape_base(device, &base);
        if (rc0 != MPGOS_OK) return cleanup(rc0);
    }
    if ((e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&s->sync_event, cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaEventCreate(&s->timer_begin)) != cudaSuccess || (e = cudaEventCreate(&s->timer_end)) != cudaSuccess)
        return cleanup(fail(MPGOS_ERR_CUDA, "stream/event creation: %s", cudaGetErrorString(e)));

    const size_t p = prec(s);
    const int64_t sizes[][3] = {
        {MPGOS_TIME_DOMAIN, 2 * nt, (int64_t)p},
        {MPGOS_ACTUAL_STATE, (int64_t)sh.sd * nt, (int64_t)p},
        {MPGOS_ACTUAL_TIME, nt, (int64_t)p},
        {MPGOS_CONTROL_PARAMETERS, (int64_t)sh.ncp * nt, (int64_t)p},
        {MPGOS_SHARED_PARAMETERS, sh.nsp, (int64_t)p},
        {MPGOS_INTEGER_SHARED_PARAMETERS, sh.nisp, 4},
        {MPGOS_ACCESSORIES, (int64_t)sh.na * nt, (int64_t)p},
        {MPGOS_INTEGER_ACCESSORIES, (int64_t)sh.nia * nt, 4},
        {MPGOS_DENSE_INDEX, nt, 4},
        {MPGOS_DENSE_TIME, (int64_t)ndo * nt, (int64_t)p},
        {MPGOS_DENSE_STATE, (int64_t)ndo * sh.sd * nt, (int64_t)p},
        {MPGOS_STATUS, nt, 4},
        {MPGOS_ACCEPTED_STEPS, nt, 4},
        {MPGOS_REJECTED_STEPS, nt, 4},
    };
    for (const auto& row : sizes) {
        Buffer& b = s->var[row[0]];
        b.count = row[1];
        b.elem = static_cast<size_t>(row[2]);
        const size_t bytes = std::max<size_t>(b.bytes(), 16);  // zero-sized arrays still get a valid pointer
        if (cudaMallocHost(&b.host, bytes) != cudaSuccess)
            return cleanup(fail(MPGOS_ERR_MEMORY, "pinned host allocation of %zu bytes failed", bytes));
        std::memset(b.host, 0, bytes);
        if (cudaMalloc(&b.device, bytes) != cudaSuccess)
            return cleanup(fail(MPGOS_ERR_MEMORY, "device allocation of %zu bytes failed", bytes));
        if (cudaMemset(b.device, 0, bytes) != cudaSuccess)
            return cleanup(fail(MPGOS_ERR_CUDA, "device memset failed"));
    }
    auto dalloc = [&](void** ptr, size_t bytes) -> bool {
        bytes = std::max<size_t>(bytes, 16);
        return cudaMalloc(ptr, bytes) == cudaSuccess && cudaMemset(*ptr, 0, bytes) == cudaSuccess;
    };
    if (!dalloc(&s->d_rtol, p * sh.sd) || !dalloc(&s->d_atol, p * sh.sd) || !dalloc(&s->d_etol, p * sh.ne) ||
        !dalloc(reinterpret_cast<void**>(&s->d_edir), 4 * sh.ne) || !dalloc(reinterpret_cast<void**>(&s->d_work), 4))
        return cleanup(fail(MPGOS_ERR_MEMORY, "device allocation of option arrays failed"));
    s->rtol.assign(sh.sd, 1e-8);
    s->atol.assign(sh.sd, 1e-8);
    s->etol.assign(sh.ne, 1e-6);
    s->edir.assign(sh.ne, 0);
    int rc = push_option_arrays(s);
    if (rc != MPGOS_OK) return cleanup(rc);
    *out = s;
    return MPGOS_OK;
}

MPGOS_EXPORT int mpgos_pt_destroy(mpgos_pt_solver* s)
{
    if (s == nullptr) return MPGOS_OK;
    cudaSetDevice(s->device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    clear_graphs(s);
    for (Buffer& b : s->var) {
        if (b.host) cudaFreeHost(b.host);
        if (b.device) cudaFree(b.device);
    }
    for (void* p : {s->d_rtol, s->d_atol, s->d_etol, static_cast<void*>(s->d_edir), static_cast<void*>(s->d_work),
                    static_cast<void*>(s->d_order), static_cast<void*>(s->d_order_scratch)})
        if (p) cudaFree(p);
    for (void* p : s->checkpoint)
        if (p) cudaFree(p);
    for (void* p : {static_cast<void*>(s->tape.dt), static_cast<void*>(s->tape.ckpt_x),
                    static_cast<void*>(s->tape.ckpt_t), static_cast<void*>(s->tape.n_steps)})
        if (p) cudaFree(p);
    if (s->timer_begin) cudaEventDestroy(s->timer_begin);
    if (s->timer_end) cudaEventDestroy(s->timer_end);
    if (s->sync_event) cudaEventDestroy(s->sync_event);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return MPGOS_OK;
}

MPGOS_EXPORT int mpgos_pt_get_shape(const mpgos_pt_solver* s, mpgos_pt_shape* shape, int64_t* nt, int32_t* ndo)
{
    int rc = check_solver(s);
    if (rc) return rc;
    if (shape) *shape = s->shape;
    if (nt) *nt = s->nt;
    if (ndo) *ndo = s->ndo;
    return MPGOS_OK;
}

MPGOS_EXPORT int mpgos_pt_set_option(mpgos_pt_solver* s, int32_t option, int32_t index, double value)
{
    int rc = check_solver(s);
    if (rc) return rc;
    g_last_error.clear();
    auto bound = [&](const char* name, int32_t limit) -> int {
        if (index < 0 || index >= limit)
            return fail(MPGOS_ERR_ARGUMENT, "SolverOption %s: index %d outside 0..%d", name, index, limit - 1);
        return MPGOS_OK;
    };
    auto positive = [&](const char* name) -> int {
        if (!(value > 0.0) || !std::isfinite(value))
            return fail(MPGOS_ERR_ARGUMENT, "SolverOption %s: value %g must be positive and finite", name, value);
        return MPGOS_OK;
    };
    switch (option) {
        case MPGOS_THREADS_PER_BLOCK: {
            const int b = static_cast<int>(value);
            if (b < 1 || b > 256 || b != value)
                return fail(MPGOS_ERR_ARGUMENT, "ThreadsPerBlock %g outside 1..256", value);
            s->block = b;
            break;
        }
        case MPGOS_INITIAL_TIME_STEP:
            if ((rc = positive("InitialTimeStep"))) return rc;
            s->initial_dt = value;
            break;
        case MPGOS_ACTIVE_NUMBER_OF_THREADS: {
            const int64_t n = static_cast<int64_t>(value);
            if (n < 0 || n > s->nt || n != value)
                return fail(MPGOS_ERR_ARGUMENT, "ActiveNumberOfThreads %g outside 0..%lld", value, (long long)s->nt);
            s->n_active = n;
            break;
        }
        case MPGOS_MAXIMUM_TIME_STEP:
            if ((rc = positive("MaximumTimeStep"))) return rc;
            s->max_dt = value;
            break;
        case MPGOS_MINIMUM_TIME_STEP:
            if ((rc = positive("MinimumTimeStep"))) return rc;
            s->min_dt = value;
            break;
        case MPGOS_TIME_STEP_GROW_LIMIT:
            if ((rc = positive("TimeStepGrowLimit"))) return rc;
            s->grow = value;
            break;
        case MPGOS_TIME_STEP_SHRINK_LIMIT:
            if ((rc = positive("TimeStepShrinkLimit"))) return rc;
            s->shrink = value;
            break;
        case MPGOS_DENSE_OUTPUT_MINIMUM_TIME_STEP:
            if (!(value >= 0.0) || !std::isfinite(value))
                return fail(MPGOS_ERR_ARGUMENT, "DenseOutputMinimumTimeStep %g must be >= 0", value);
            s->dense_min_dt = value;
            break;
        case MPGOS_DENSE_OUTPUT_SAVE_FREQUENCY: {
            const int f = static_cast<int>(value);
            if (f < 1 || f != value) return fail(MPGOS_ERR_ARGUMENT, "DenseOutputSaveFrequency %g must be >= 1", value);
            s->dense_freq = f;
            break;
        }
        case MPGOS_PREFER_SHARED_MEMORY:
            s->prefer_shared = value != 0.0 ? 1 : 0;
            break;
        case MPGOS_RELATIVE_TOLERANCE:
        case MPGOS_ABSOLUTE_TOLERANCE:
            if ((rc = bound(option == MPGOS_RELATIVE_TOLERANCE ? "RelativeTolerance" : "AbsoluteTolerance", s->shape.sd))) return rc;
            if (!(value >= 0.0) || !std::isfinite(value))
                return fail(MPGOS_ERR_ARGUMENT, "tolerance %g must be finite and >= 0", value);
            (option == MPGOS_RELATIVE_TOLERANCE ? s->rtol : s->atol)[index] = value;
            if ((rc = push_option_arrays(s))) return rc;
            break;
        case MPGOS_EVENT_TOLERANCE:
            if ((rc = bound("EventTolerance", s->shape.ne))) return rc;
            if (!(value >= 0.0) || !std::isfinite(value))
                return fail(MPGOS_ERR_ARGUMENT, "EventTolerance %g must be finite and >= 0", value);
            s->etol[index] = value;
            if ((rc = push_option_arrays(s))) return rc;
            break;
        case MPGOS_EVENT_DIRECTION:
            if ((rc = bound("EventDirection", s->shape.ne))) return rc;
            s->edir[index] = static_cast<int32_t>(value);
            if ((rc = push_option_arrays(s))) return rc;
            break;
        case MPGOS_KERNEL_MODE: {
            const int32_t m = static_cast<int32_t>(value);
            if (m < 0 || (m & ~(MPGOS_MODE_FAST_CONTROL | MPGOS_MODE_PERSISTENT | MPGOS_MODE_FP32_STAGE |
                                 MPGOS_MODE_DF_STAGE | MPGOS_MODE_SPLIT)) || m != value)
                return fail(MPGOS_ERR_ARGUMENT, "kernel mode %g is not a set of MPGOS_MODE_* bits", value);
            // FAST_CONTROL only changes the adaptive FP64 controller and is a
            // no-op elsewhere; FP32_STAGE and DF_STAGE change the arithmetic
            // and must exist.
            if ((m & MPGOS_MODE_FP32_STAGE) && !(s->shape.modes & MPGOS_MODE_FP32_STAGE))
                return fail(MPGOS_ERR_UNSUPPORTED, "FP32_STAGE mode not compiled for this table (modes 0x%x)", s->shape.modes);
            if ((m & MPGOS_MODE_DF_STAGE) && !(s->shape.modes & MPGOS_MODE_DF_STAGE))
                return fail(MPGOS_ERR_UNSUPPORTED, "DF_STAGE mode not compiled for this table (modes 0x%x)", s->shape.modes);
            if ((m & MPGOS_MODE_DF_STAGE) && (m & MPGOS_MODE_FP32_STAGE))
                return fail(MPGOS_ERR_ARGUMENT, "DF_STAGE and FP32_STAGE are exclusive");
            if ((m & MPGOS_MODE_SPLIT) && !(s->shape.modes & MPGOS_MODE_SPLIT))
                return fail(MPGOS_ERR_UNSUPPORTED, "SPLIT mode not compiled for this table (modes 0x%x)", s->shape.modes);
            if ((m & MPGOS_MODE_SPLIT) && (m & (MPGOS_MODE_DF_STAGE | MPGOS_MODE_FP32_STAGE)))
                return fail(MPGOS_ERR_ARGUMENT, "SPLIT is exclusive with DF_STAGE and FP32_STAGE");
            s->mode = m;
            break;
        }
        case MPGOS_MAXIMUM_ATTEMPTS: {
            const int64_t n = static_cast<int64_t>(value);
            if (n < 1) return fail(MPGOS_ERR_ARGUMENT, "MaximumAttempts %g must be >= 1", value);
            s->max_attempts = n;
            break;
        }
        case MPGOS_INSTANCES_PER_THREAD: {
            const int32_t n = static_cast<int32_t>(value);
            if (n < 1 || n > 64 || n != value)
                return fail(MPGOS_ERR_ARGUMENT, "InstancesPerThread %g must be an integer in 1..64", value);
            s->ipt = n;
            break;
        }
        case MPGOS_WARP_RECONVERGE:
            if (value != 0.0 && value != 1.0) return fail(MPGOS_ERR_ARGUMENT, "WarpReconverge %g must be 0 or 1", value);
            s->reconverge = static_cast<int32_t>(value);
            break;
        case MPGOS_OUTLINE_RHS:
            if (value != 0.0 && value != 1.0) return fail(MPGOS_ERR_ARGUMENT, "OutlineRhs %g must be 0 or 1", value);
            s->outline = static_cast<int32_t>(value);
            break;
        case MPGOS_WORK_ORDER:
            if (value != 0.0 && value != 1.0) return fail(MPGOS_ERR_ARGUMENT, "WorkOrder %g must be 0 or 1", value);
            if (value == 1.0 && s->d_order == nullptr) {
                MPGOS_CUDA(cudaSetDevice(s->device));
                const size_t counters = static_cast<size_t>(mpgos_internal_order_scratch_counters());
                if (cudaMalloc(reinterpret_cast<void**>(&s->d_order), sizeof(int32_t) * std::max<int64_t>(s->nt, 1)) !=
                        cudaSuccess ||
                    cudaMalloc(reinterpret_cast<void**>(&s->d_order_scratch), sizeof(unsigned) * counters) !=
                        cudaSuccess) {
                    cudaFree(s->d_order);
                    s->d_order = nullptr;
                    s->d_order_scratch = nullptr;
                    return fail(MPGOS_ERR_MEMORY, "work-order buffers (%lld instances) allocation failed",
                                static_cast<long long>(s->nt));
                }
            }
            s->work_order = static_cast<int32_t>(value);
            break;
        default:
            return fail(MPGOS_ERR_ARGUMENT, "unknown solver option %d", option);
    }
    s->generation++;
    return MPGOS_OK;
}

MPGOS_EXPORT int mpgos_pt_get_option(const mpgos_pt_solver* s, int32_t option, int32_t index, double* value)
{
    int rc = check_solver(s);
    if (rc) return rc;
    if (value == nullptr) return fail(MPGOS_ERR_ARGUMENT, "null value pointer");
    auto indexed = [&](const std::vector<double>& v) -> int {
        if (index < 0 || index >= (int32_t)v.size()) return fail(MPGOS_ERR_ARGUMENT, "option index %d out of range", index);
        *value = v[index];
        return MPGOS_OK;
    };
    switch (option) {
        case MPGOS_THREADS_PER_BLOCK: *value = s->block; break;
        case MPGOS_INITIAL_TIME_STEP: *value = s->initial_dt; break;
        case MPGOS_ACTIVE_NUMBER_OF_THREADS: *value = (double)s->n_active; break;
        case MPGOS_MAXIMUM_TIME_STEP: *value = s->max_dt; break;
        case MPGOS_MINIMUM_TIME_STEP: *value = s->min_dt; break;
        case MPGOS_TIME_STEP_GROW_LIMIT: *value = s->grow; break;
        case MPGOS_TIME_STEP_SHRINK_LIMIT: *value = s->shrink; break;
        case MPGOS_DENSE_OUTPUT_MINIMUM_TIME_STEP: *value = s->dense_min_dt; break;
        case MPGOS_DENSE_OUTPUT_SAVE_FREQUENCY: *value = s->dense_freq; break;
        case MPGOS_PREFER_SHARED_MEMORY: *value = s->prefer_shared; break;
        case MPGOS_RELATIVE_TOLERANCE: return indexed(s->rtol);
        case MPGOS_ABSOLUTE_TOLERANCE: return indexed(s->atol);
        case MPGOS_EVENT_TOLERANCE: return indexed(s->etol);
        case MPGOS_EVENT_DIRECTION: {
            if (index < 0 || index >= (int32_t)s->edir.size()) return fail(MPGOS_ERR_ARGUMENT, "option index %d out of range", index);
            *value = s->edir[index];
            break;
        }
        case MPGOS_KERNEL_MODE: *value = s->mode; break;
        case MPGOS_MAXIMUM_ATTEMPTS: *value = (double)s->max_attempts; break;
        case MPGOS_INSTANCES_PER_THREAD: *value = s->ipt; break;
        case MPGOS_WARP_RECONVERGE: *value = s->reconverge >= 0 ? s->reconverge : (s->shape.ne > 0 ? 1 : 0); break;
        case MPGOS_OUTLINE_RHS: *value = s->outline; break;
        case MPGOS_WORK_ORDER: *value = s->work_order; break;
        default: return fail(MPGOS_ERR_ARGUMENT, "unknown solver option %d", option);
    }
    return MPGOS_OK;
}

MPGOS_EXPORT int mpgos_pt_host_buffer(mpgos_pt_solver* s, int32_t variable, void** ptr, int64_t* count)
{
    int rc = check_solver(s);
    if (rc) return rc;
    if (!(is_reference_variable(variable) || is_extension_variable(variable)))
        return fail(MPGOS_ERR_ARGUMENT, "variable %d has no single host buffer", variable);
    if (ptr) *ptr = s->var[variable].host;
    if (count) *count = s->var[variable].count;
    return MPGOS_OK;
}

MPGOS_EXPORT int mpgos_pt_device_buffer(mpgos_pt_solver* s, int32_t variable, void** ptr, int64_t* count)
{
    int rc = check_solver(s);
    if (rc) return rc;
    if (!(is_reference_variable(variable) || is_extension_variable(variable)))
        return fail(MPGOS_ERR_ARGUMENT, "variable %d has no single device buffer", variable);
    if (ptr) *ptr = s->var[variable].device;
    if (count) *count = s->var[variable].count;
    return MPGOS_OK;
}

namespace {
// Variables moved by one Synchronise call (SingleSystem_PerThread_Interface.cuh:833-965).
std::vector<int32_t> expand_variable(int32_t v)
{
    if (v == MPGOS_ALL)
        return {MPGOS_TIME_DOMAIN, MPGOS_ACTUAL_STATE, MPGOS_ACTUAL_TIME, MPGOS_CONTROL_PARAMETERS,
                MPGOS_SHARED_PARAMETERS, MPGOS_ACCESSORIES, MPGOS_INTEGER_SHARED_PARAMETERS,
                MPGOS_INTEGER_ACCESSORIES, MPGOS_DENSE_INDEX, MPGOS_DENSE_TIME, MPGOS_DENSE_STATE};
    if (v == MPGOS_DENSE_OUTPUT) return {MPGOS_DENSE_INDEX, MPGOS_DENSE_TIME, MPGOS_DENSE_STATE};
    if (v == MPGOS_TIME_DOMAIN || v == MPGOS_ACTUAL_STATE || v == MPGOS_ACTUAL_TIME || v == MPGOS_CONTROL_PARAMETERS ||
        v == MPGOS_SHARED_PARAMETERS || v == MPGOS_INTEGER_SHARED_PARAMETERS || v == MPGOS_ACCESSORIES ||
        v == MPGOS_INTEGER_ACCESSORIES || is_extension_variable(v))
        return {v};
    return {};
}
}  // namespace

MPGOS_EXPORT int mpgos_pt_sync_h2d(mpgos_pt_solver* s, int32_t variable)
{
    int rc = check_solver(s);
    if (rc) return rc;
    std::vector<int32_t> vs = expand_variable(variable);
    if (vs.empty()) return fail(MPGOS_ERR_ARGUMENT, "SynchroniseFromHostToDevice: variable %d not applicable", variable);
    MPGOS_CUDA(cudaSetDevice(s->device));
    for (int32_t v : vs) {
        const Buffer& b = s->var[v];
        if (b.bytes() > 0) MPGOS_CUDA(cudaMemcpyAsync(b.device, b.host, b.bytes(), cudaMemcpyHostToDevice, s->stream));
    }
    return MPGOS_OK;
}

MPGOS_EXPORT int mpgos_pt_sync_d2h(mpgos_pt_solver* s, int32_t variable)
{
    int rc = check_solver(s);
    if (rc) return rc;
    std::vector<int32_t> vs = expand_variable(variable);
    if (vs.empty()) return fail(MPGOS_ERR_ARGUMENT, "SynchroniseFromDeviceToHost: variable %d not applicable", variable);
    MPGOS_CUDA(cudaSetDevice(s->device));
    for (int32_t v : vs) {
        const Buffer& b = s->var[v];
        if (b.bytes() > 0) MPGOS_CUDA(cudaMemcpyAsync(b.host, b.device, b.bytes(), cudaMemcpyDeviceToHost, s->stream));
    }
    return MPGOS_OK;
}

MPGOS_EXPORT int mpgos_pt_solve(mpgos_pt_solver* s)
{
    int rc = check_solver(s);
    if (rc) return rc;
    MPGOS_CUDA(cudaSetDevice(s->device));
    return enqueue_solve(s, s->mode, s->block);
}

MPGOS_EXPORT int mpgos_pt_solve_phases(mpgos_pt_solver* s, int32_t n_phases, int32_t stream_accessory, void* phase_output)
{
    int rc = check_solver(s);
    if (rc) return rc;
    if (n_phases < 0) return fail(MPGOS_ERR_ARGUMENT, "negative number of phases");
    if (stream_accessory >= 0) {
        if (stream_accessory >= s->shape.na)
            return fail(MPGOS_ERR_ARGUMENT, "stream_accessory %d outside 0..%d", stream_accessory, s->shape.na - 1);
        if (phase_output == nullptr) return fail(MPGOS_ERR_ARGUMENT, "null phase_output");
    }
    if (n_phases == 0 || s->n_active <= 0) return MPGOS_OK;
    MPGOS_CUDA(cudaSetDevice(s->device));
    GraphKey key{n_phases, stream_accessory, phase_output, s->generation};
    auto it = s->graphs.find(key);
    if (it == s->graphs.end()) {
        // Drop graphs of older option generations before building a new one.
        for (auto g = s->graphs.begin(); g != s->graphs.end();) {
            if (g->first.generation != s->generation) {
                cudaGraphExecDestroy(g->second);
                g = s->graphs.erase(g);
            } else {
                ++g;
            }
        }
        const size_t col_bytes = prec(s) * static_cast<size_t>(s->nt);
        const char* acc_dev = static_cast<const char*>(s->var[MPGOS_ACCESSORIES].device);
        MPGOS_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
        int crc = MPGOS_OK;
        for (int32_t p = 0; p < n_phases && crc == MPGOS_OK; p++) {
            crc = enqueue_solve(s, s->mode, s->block);
            if (crc == MPGOS_OK && stream_accessory >= 0) {
                cudaError_t e = cudaMemcpyAsync(static_cast<char*>(phase_output) + col_bytes * p,
                                                acc_dev + col_bytes * stream_accessory, col_bytes,
                                                cudaMemcpyDeviceToDevice, s->stream);
                if (e != cudaSuccess) crc = fail(MPGOS_ERR_CUDA, "phase output copy: %s", cudaGetErrorString(e));
            }
        }
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamEndCapture(s->stream, &graph);
        if (crc != MPGOS_OK) {
            if (graph) cudaGraphDestroy(graph);
            return crc;
        }
        if (e != cudaSuccess) return fail(MPGOS_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
        cudaGraphExec_t exec = nullptr;
        e = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return fail(MPGOS_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
        it = s->graphs.emplace(key, exec).first;
    }
    MPGOS_CUDA(cudaGraphLaunch(it->second, s->stream));
    return MPGOS_OK;
}

MPGOS_EXPORT int mpgos_pt_insert_sync_point(mpgos_pt_solver* s)
{
    int rc = check_solver(s);
    if (rc) return rc;
    MPGOS_CUDA(cudaSetDevice(s->device));
    MPGOS_CUDA(cudaEventRecord(s->sync_event, s->stream));
    return MPGOS_OK;
}

MPGOS_EXPORT int mpgos_pt_sync_solver(mpgos_pt_solver* s)
{
    int rc = check_solver(s);
    if (rc) return rc;
    MPGOS_CUDA(cudaSetDevice(s->device));
    MPGOS_CUDA(cudaEventSynchronize(s->sync_event));
    MPGOS_CUDA(cudaGetLastError());
    return MPGOS_OK;
}

MPGOS_EXPORT int mpgos_pt_sync_device(mpgos_pt_solver* s)
{
    int rc = check_solver(s);
    if (rc) return rc;
    MPGOS_CUDA(cudaSetDevice(s->device));
    MPGOS_CUDA(cudaDeviceSynchronize());
    return MPGOS_OK;
}

MPGOS_EXPORT int mpgos_pt_stream(mpgos_pt_solver* s, void** stream)
{
    int rc = check_solver(s);
    if (rc) return rc;
    if (stream) *stream = s->stream;
    return MPGOS_OK;
}

MPGOS_EXPORT int mpgos_pt_launch_config(mpgos_pt_solver* s, int* grid, int* block, int32_t* mode)
{
    int rc = check_solver(s);
    if (rc) return rc;
    const int32_t m = effective_mode(s, s->mode);
    int g = 0;
    if (s->n_active > 0 && (rc = grid_for(s, m, s->block, &g))) return rc;
    if (grid) *grid = g;
    if (block) *block = s->block;
    if (mode) *mode = m;
    return MPGOS_OK;
}

MPGOS_EXPORT int mpgos_pt_timer_start(mpgos_pt_solver* s)
{
    int rc = check_solver(s);
    if (rc) return rc;
    MPGOS_CUDA(cudaSetDevice(s->device));
    MPGOS_CUDA(cudaEventRecord(s->timer_begin, s->stream));
    return MPGOS_OK;
}

MPGOS_EXPORT int mpgos_pt_timer_stop(mpgos_pt_solver* s, float* ms)
{
    int rc = check_solver(s);
    if (rc) return rc;
    MPGOS_CUDA(cudaSetDevice(s->device));
    MPGOS_CUDA(cudaEventRecord(s->timer_end, s->stream));
    MPGOS_CUDA(cudaEventSynchronize(s->timer_end));
    float t = 0.f;
    MPGOS_CUDA(cudaEventElapsedTime(&t, s->timer_begin, s->timer_end));
    if (ms) *ms = t;
    return MPGOS_OK;
}

MPGOS_EXPORT int mpgos_pt_autotune(mpgos_pt_solver* s, int32_t arithmetic, const char* cache_path)
{
    int rc = check_solver(s);
    if (rc) return rc;
    if (s->n_active <= 0) return MPGOS_OK;
    MPGOS_CUDA(cudaSetDevice(s->device));
    int32_t base = 0;
    if ((arithmetic & MPGOS_MODE_SPLIT) && (s->shape.modes & MPGOS_MODE_SPLIT))
        base = MPGOS_MODE_SPLIT;
    else if ((arithmetic & MPGOS_MODE_DF_STAGE) && (s->shape.modes & MPGOS_MODE_DF_STAGE))
        base = MPGOS_MODE_DF_STAGE;
    else if (arithmetic && (s->shape.modes & MPGOS_MODE_FAST_CONTROL))
        base = MPGOS_MODE_FAST_CONTROL;

    std::ostringstream key;
    key << s->k->name << "/sd" << s->shape.sd << "/alg" << s->shape.algorithm << "/p" << s->shape.precision_bytes
        << "/nt" << s->n_active << "/ndo" << s->ndo << "/m" << base << "/" << s->gpu_name;
    const std::string k = key.str();

    // Cached choice?
    if (cache_path != nullptr) {
        std::ifstream in(cache_path);
        std::string line;
        while (std::getline(in, line)) {
            const std::string tag = "\"" + json_escape(k) + "\"";
            size_t pos = line.find(tag);
            if (pos == std::string::npos) continue;
            int b = 0, m = 0, n = 1, ps = s->prefer_shared, rv = s->reconverge, ol = 0;
            const char* bp = std::strstr(line.c_str() + pos, "\"block\":");
            const char* mp = std::strstr(line.c_str() + pos, "\"mode\":");
            const char* np = std::strstr(line.c_str() + pos, "\"instances_per_thread\":");
            const char* pp = std::strstr(line.c_str() + pos, "\"prefer_shared\":");
            const char* rp = std::strstr(line.c_str() + pos, "\"reconverge\":");
            const char* op = std::strstr(line.c_str() + pos, "\"outline_rhs\":");
            if (np) sscanf(np, "\"instances_per_thread\": %d", &n);
            if (pp) sscanf(pp, "\"prefer_shared\": %d", &ps);
            if (rp) sscanf(rp, "\"reconverge\": %d", &rv);
            if (op) sscanf(op, "\"outline_rhs\": %d", &ol);
            if (bp && mp && sscanf(bp, "\"block\": %d", &b) == 1 && sscanf(mp, "\"mode\": %d", &m) == 1 && b >= 1 &&
                b <= 256 && n >= 1 && n <= 64) {
                s->block = b;
                s->mode = m;
                s->ipt = n;
                s->prefer_shared = ps ? 1 : 0;
                s->reconverge = (rv == 0 || rv == 1) ? rv : -1;
                s->outline = ol ? 1 : 0;
                s->generation++;
                return MPGOS_OK;
            }
        }
    }

    // Back up every array a launch writes, try each candidate, restore.
    const int32_t mutable_vars[] = {MPGOS_TIME_DOMAIN, MPGOS_ACTUAL_STATE, MPGOS_ACTUAL_TIME, MPGOS_CONTROL_PARAMETERS,
                                    MPGOS_ACCESSORIES, MPGOS_INTEGER_ACCESSORIES, MPGOS_DENSE_INDEX,
                                    MPGOS_DENSE_TIME, MPGOS_DENSE_STATE};
    std::vector<void*> backup;
    auto release = [&]() {
        for (void* p : backup)
            if (p) cudaFree(p);
    };
    for (int32_t v : mutable_vars) {
        void* p = nullptr;
        const size_t bytes = std::max<size_t>(s->var[v].bytes(), 16);
        if (cudaMalloc(&p, bytes) != cudaSuccess) {
            release();
            return fail(MPGOS_ERR_MEMORY, "autotune backup allocation failed");
        }
        backup.push_back(p);
        if (cudaMemcpyAsync(p, s->var[v].device, bytes, cudaMemcpyDeviceToDevice, s->stream) != cudaSuccess) {
            release();
            return fail(MPGOS_ERR_CUDA, "autotune backup copy failed");
        }
    }
    auto restore = [&]() -> int {
        for (size_t i = 0; i < backup.size(); i++) {
            const int32_t v = mutable_vars[i];
            const size_t bytes = std::max<size_t>(s->var[v].bytes(), 16);
            MPGOS_CUDA(cudaMemcpyAsync(s->var[v].device, backup[i], bytes, cudaMemcpyDeviceToDevice, s->stream));
        }
        return MPGOS_OK;
    };

    // Candidates: block size x mapping (static with 1, 2 or 4 instances per
    // thread, or persistent) x placement of the shared parameters (shared
    // memory or global loads; only where the system has any).
    float best = 1e30f;
    int best_block = s->block, best_ipt = s->ipt, best_ps = s->prefer_shared;
    int32_t best_mode = s->mode;
    const int keep_ipt = s->ipt, keep_ps = s->prefer_shared;
    // one timed Solve() from the backed-up state; errors are returned (not
    // thrown out of the tuner) so that the state and the backups are restored
    auto time_one = [&](int32_t m, int b, float* ms) -> int {
        int r = restore();
        if (r) return r;
        cudaError_t e = cudaEventRecord(s->timer_begin, s->stream);
        if (e == cudaSuccess && (r = enqueue_solve(s, m, b))) return r;
        if (e == cudaSuccess) e = cudaEventRecord(s->timer_end, s->stream);
        if (e == cudaSuccess) e = cudaEventSynchronize(s->timer_end);
        if (e == cudaSuccess) e = cudaEventElapsedTime(ms, s->timer_begin, s->timer_end);
        if (e != cudaSuccess) return fail(MPGOS_ERR_CUDA, "autotune timing failed: %s", cudaGetErrorString(e));
        return MPGOS_OK;
    };
    const int blocks[] = {32, 64, 96, 128, 192, 256};
    const int ipts[] = {1, 2, 4, 0};  // 0: persistent
    const bool has_shared = (s->shape.nsp + s->shape.nisp) > 0;
    // double-float kernels: every candidate with the right-hand side inlined
    // and out of line (the best mapping differs between the two)
    const int keep_ol = s->outline;
    int best_ol = keep_ol;
    const bool df_base = (effective_mode(s, base) & (MPGOS_MODE_DF_STAGE | MPGOS_MODE_SPLIT)) != 0;
    for (int ol = df_base ? 0 : keep_ol; ol <= (df_base ? 1 : keep_ol) && !rc; ol++) {
        s->outline = ol;
        for (int ps = has_shared ? 0 : keep_ps; ps <= (has_shared ? 1 : keep_ps); ps++) {
            for (int n : ipts) {
                for (int b : blocks) {
                    const int32_t m = base | (n == 0 ? MPGOS_MODE_PERSISTENT : 0);
                    s->ipt = n == 0 ? 1 : n;
                    s->prefer_shared = ps;
                    float t = 0.f;
                    if ((rc = time_one(m, b, &t))) break;
                    if (t < best) {
                        best = t;
                        best_block = b;
                        best_mode = m;
                        best_ipt = s->ipt;
                        best_ps = ps;
                        best_ol = ol;
                    }
                }
                if (rc) break;
            }
            if (rc) break;
        }
    }
    s->outline = best_ol;
    // the warp reconvergence ballot, on and off, at the best configuration
    const int keep_rv = s->reconverge;
    const int cur_rv = keep_rv >= 0 ? keep_rv : (s->shape.ne > 0 ? 1 : 0);
    int best_rv = cur_rv;
    if (!rc) {
        s->ipt = best_ipt;
        s->prefer_shared = best_ps;
        s->reconverge = 1 - cur_rv;
        float t = 0.f;
        if (!(rc = time_one(best_mode, best_block, &t)) && t < best) {
            best = t;
            best_rv = 1 - cur_rv;
        }
    }
    s->outline = keep_ol;
    s->reconverge = keep_rv;
    s->ipt = keep_ipt;
    s->prefer_shared = keep_ps;
    if (rc) {
        restore();
        cudaStreamSynchronize(s->stream);
        release();
        return rc;
    }
    rc = restore();
    cudaStreamSynchronize(s->stream);
    release();
    if (rc) return rc;
    s->block = best_block;
    s->mode = best_mode;
    s->ipt = best_ipt;
    s->prefer_shared = best_ps;
    s->reconverge = best_rv;
    s->outline = best_ol;
    s->generation++;

    if (cache_path != nullptr) {
        std::ofstream outf(cache_path, std::ios::app);
        if (outf) outf << "{\"" << json_escape(k) << "\": {\"block\": " << best_block << ", \"mode\": " << best_mode
                       << ", \"instances_per_thread\": " << best_ipt << ", \"prefer_shared\": " << best_ps
                       << ", \"reconverge\": " << best_rv << ", \"outline_rhs\": " << best_ol << ", \"ms\": " << best
                       << "}}\n";
    }
    return MPGOS_OK;
}

namespace {
// Arrays a launch may write (SingleSystem_PerThread_Solver.cuh:414-435 plus dense output).
const int32_t kCheckpointVars[] = {MPGOS_TIME_DOMAIN, MPGOS_ACTUAL_STATE, MPGOS_ACTUAL_TIME, MPGOS_CONTROL_PARAMETERS,
                                   MPGOS_ACCESSORIES, MPGOS_INTEGER_ACCESSORIES, MPGOS_DENSE_INDEX,
                                   MPGOS_DENSE_TIME, MPGOS_DENSE_STATE};
}  // namespace

MPGOS_EXPORT int mpgos_pt_checkpoint_save(mpgos_pt_solver* s)
{
    int rc = check_solver(s);
    if (rc) return rc;
    MPGOS_CUDA(cudaSetDevice(s->device));
    const size_t n = sizeof(kCheckpointVars) / sizeof(kCheckpointVars[0]);
    if (s->checkpoint.empty()) {
        s->checkpoint.assign(n, nullptr);
        for (size_t i = 0; i < n; i++) {
            const size_t bytes = std::max<size_t>(s->var[kCheckpointVars[i]].bytes(), 16);
            if (cudaMalloc(&s->checkpoint[i], bytes) != cudaSuccess)
                return fail(MPGOS_ERR_MEMORY, "checkpoint allocation of %zu bytes failed", bytes);
        }
    }
    for (size_t i = 0; i < n; i++) {
        const Buffer& b = s->var[kCheckpointVars[i]];
        if (b.bytes()) MPGOS_CUDA(cudaMemcpyAsync(s->checkpoint[i], b.device, b.bytes(), cudaMemcpyDeviceToDevice, s->stream));
    }
    return MPGOS_OK;
}

MPGOS_EXPORT int mpgos_pt_checkpoint_restore(mpgos_pt_solver* s)
{
    int rc = check_solver(s);
    if (rc) return rc;
    if (s->checkpoint.empty()) return fail(MPGOS_ERR_ARGUMENT, "no checkpoint saved");
    MPGOS_CUDA(cudaSetDevice(s->device));
    const size_t n = sizeof(kCheckpointVars) / sizeof(kCheckpointVars[0]);
    for (size_t i = 0; i < n; i++) {
        const Buffer& b = s->var[kCheckpointVars[i]];
        if (b.bytes()) MPGOS_CUDA(cudaMemcpyAsync(b.device, s->checkpoint[i], b.bytes(), cudaMemcpyDeviceToDevice, s->stream));
    }
    return MPGOS_OK;
}

// ---- discrete adjoint -----------------------------------------------------------
MPGOS_EXPORT int mpgos_pt_solve_record(mpgos_pt_solver* s, int32_t max_steps, int32_t segment)
{
    int rc = check_solver(s);
    if (rc) return rc;
    if (s->k->launch_record == nullptr || s->shape.precision_bytes != 8)
        return fail(MPGOS_ERR_UNSUPPORTED, "system %s has no adjoint kernels compiled (FP64 only)", s->k->name);
    if (max_steps < 1 || segment < 1 || segment > 64)
        return fail(MPGOS_ERR_ARGUMENT, "tape: max_steps %d must be >= 1 and segment %d within 1..64", max_steps, segment);
    // from here on the reverse pass reads this call's tape (or, if this call
    // fails, none that a later static recording did not write)
    s->use_static_tape = false;
    MPGOS_CUDA(cudaSetDevice(s->device));
    const size_t nt = static_cast<size_t>(s->nt), sd = static_cast<size_t>(s->shape.sd);
    const size_t nck = static_cast<size_t>(max_steps / segment + 1);
    if (s->tape.max_steps != max_steps || s->tape.segment != segment || s->tape.dt == nullptr) {
        MPGOS_CUDA(cudaStreamSynchronize(s->stream));
        for (void* p : {static_cast<void*>(s->tape.dt), static_cast<void*>(s->tape.ckpt_x),
                        static_cast<void*>(s->tape.ckpt_t), static_cast<void*>(s->tape.n_steps)})
            if (p) cudaFree(p);
        s->tape = mpgos_pt_tape{};
        const size_t b_dt = static_cast<size_t>(max_steps) * nt * 8, b_cx = nck * sd * nt * 8, b_ct = nck * nt * 8;
        if (cudaMalloc(reinterpret_cast<void**>(&s->tape.dt), b_dt) != cudaSuccess ||
            cudaMalloc(reinterpret_cast<void**>(&s->tape.ckpt_x), b_cx) != cudaSuccess ||
            cudaMalloc(reinterpret_cast<void**>(&s->tape.ckpt_t), b_ct) != cudaSuccess ||
            cudaMalloc(reinterpret_cast<void**>(&s->tape.n_steps), nt * 4) != cudaSuccess) {
            s->tape.max_steps = 0;
            return fail(MPGOS_ERR_MEMORY, "adjoint tape allocation (%zu bytes) failed", b_dt + b_cx + b_ct + nt * 4);
        }
        s->tape.max_steps = max_steps;
        s->tape.segment = segment;
        s->tape_bytes = b_dt + b_cx + b_ct + nt * 4;
    }
    if (s->n_active <= 0) return MPGOS_OK;
    const int32_t m = effective_mode(s, s->mode) & (MPGOS_MODE_FAST_CONTROL | MPGOS_MODE_PERSISTENT | MPGOS_MODE_DF_STAGE |
                                                   MPGOS_MODE_SPLIT);
    int grid = 0;
    if ((rc = grid_for(s, m, s->block, &grid))) return rc;
    if (m & MPGOS_MODE_PERSISTENT) MPGOS_CUDA(cudaMemsetAsync(s->d_work, 0, sizeof(uint32_t), s->stream));
    mpgos_pt_launch L;
    fill_launch(s, L, m);
    rc = s->k->launch_record(&L, &s->tape, grid, s->block, dynamic_smem(s), s->stream);
    if (rc != 0) return fail(MPGOS_ERR_CUDA, "recording launch failed: %s", cudaGetErrorString((cudaError_t)rc));
    return MPGOS_OK;
}

MPGOS_EXPORT int mpgos_pt_adjoint(mpgos_pt_solver* s, const double* dLdxT, double* dLdx0, double* dLdp)
{
    int rc = check_solver(s);
    if (rc) return rc;
    if (s->k->launch_adjoint == nullptr) return fail(MPGOS_ERR_UNSUPPORTED, "system %s has no adjoint kernels", s->k->name);
    const mpgos_pt_tape& tape = s->use_static_tape ? s->static_tape : s->tape;
    if (tape.dt == nullptr) return fail(MPGOS_ERR_ARGUMENT, "no recorded forward pass (call mpgos_pt_solve_record first)");
    if (dLdxT == nullptr || dLdx0 == nullptr || (dLdp == nullptr && s->shape.ncp > 0))
        return fail(MPGOS_ERR_ARGUMENT, "null gradient buffer");
    if (s->n_active <= 0) return MPGOS_OK;
    MPGOS_CUDA(cudaSetDevice(s->device));
    const int block = 64;
    const int64_t grid = (s->n_active + block - 1) / block;
    mpgos_pt_launch L;
    // the reverse pass computes in double-float when the solver does
    fill_launch(s, L, effective_mode(s, s->mode) & (MPGOS_MODE_DF_STAGE | MPGOS_MODE_SPLIT));
    rc = s->k->launch_adjoint(&L, &tape, dLdxT, dLdx0, dLdp, static_cast<int>(grid), block, dynamic_smem(s), s->stream);
    if (rc != 0) return fail(MPGOS_ERR_CUDA, "adjoint launch failed: %s", cudaGetErrorString((cudaError_t)rc));
    return MPGOS_OK;
}

MPGOS_EXPORT int mpgos_pt_dense_interpolate(mpgos_pt_solver* s, const double* times, int32_t n_times, double* out)
{
    int rc = check_solver(s);
    if (rc) return rc;
    if (s->k->dense_interpolate == nullptr)
        return fail(MPGOS_ERR_UNSUPPORTED, "system %s has no dense-output interpolation kernel", s->k->name);
    if (s->ndo < 1) return fail(MPGOS_ERR_ARGUMENT, "dense-output interpolation needs NDO > 0 (this object has 0)");
    if (n_times < 0 || (n_times > 0 && (times == nullptr || out == nullptr)))
        return fail(MPGOS_ERR_ARGUMENT, "dense-output interpolation: %d times, times %p, out %p", n_times,
                    static_cast<const void*>(times), static_cast<void*>(out));
    if (n_times == 0 || s->n_active <= 0) return MPGOS_OK;
    MPGOS_CUDA(cudaSetDevice(s->device));
    const int block = 128;
    const int64_t grid = (s->n_active + block - 1) / block;
    mpgos_pt_launch L;
    fill_launch(s, L, 0);
    rc = s->k->dense_interpolate(&L, times, n_times, out, static_cast<int>(grid), block, dynamic_smem(s), s->stream);
    if (rc != 0) return fail(MPGOS_ERR_CUDA, "dense interpolation launch failed: %s", cudaGetErrorString((cudaError_t)rc));
    return MPGOS_OK;
}

MPGOS_EXPORT int mpgos_pt_tape_info(const mpgos_pt_solver* s, mpgos_pt_tape* tape)
{
    int rc = check_solver(s);
    if (rc) return rc;
    if (tape == nullptr) return fail(MPGOS_ERR_ARGUMENT, "null tape pointer");
    *tape = s->use_static_tape ? s->static_tape : s->tape;
    return MPGOS_OK;
}

// ---- recording into static device scratch ------------------------------------
// The tape of mpgos_pt_solve_record_static lives in this file-scope device
// array instead of cudaMalloc'd buffers: [dt][ckpt_x][ckpt_t][n_steps], each
// part starting on a 256-byte boundary.
static __device__ __align__(256) unsigned char g_static_tape[MPGOS_STATIC_TAPE_BYTES];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_static_tape_mu;
void* g_static_tape_addr[kMaxDevices] = {};

size_t align256(size_t b) { return (b + 255) / 256 * 256; }

// Device address of g_static_tape on the current device, looked up once per
// device ordinal at the first solver creation on it (the lookup loads this
// library's device module, which reserves the array). The cached address
// belongs to the device's primary context: it is stale after
// cudaDeviceReset, which the static entry point therefore does not support.
int static_tape_base(int device, unsigned char** base)
{
    if (device < 0 || device >= kMaxDevices) return fail(MPGOS_ERR_ARGUMENT, "device ordinal %d out of range", device);
    std::lock_guard<std::mutex> lock(g_static_tape_mu);
    if (g_static_tape_addr[device] == nullptr) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_static_tape);
        if (e != cudaSuccess || p == nullptr)
            return fail(MPGOS_ERR_CUDA, "cudaGetSymbolAddress(static tape) on device %d failed: %s", device,
                        cudaGetErrorString(e));
        g_static_tape_addr[device] = p;
    }
    *base = static_cast<unsigned char*>(g_static_tape_addr[device]);
    return MPGOS_OK;
}
}  // namespace

MPGOS_EXPORT int mpgos_pt_solve_record_static(mpgos_pt_solver* s, int32_t max_steps, int32_t segment)
{
    int rc = check_solver(s);
    if (rc) return rc;
    if (s->k->launch_record == nullptr || s->shape.precision_bytes != 8)
        return fail(MPGOS_ERR_UNSUPPORTED, "system %s has no adjoint kernels compiled (FP64 only)", s->k->name);
    if (max_steps < 1 || segment < 1 || segment > 64)
        return fail(MPGOS_ERR_ARGUMENT, "tape: max_steps %d must be >= 1 and segment %d within 1..64", max_steps, segment);
    const size_t nt = static_cast<size_t>(s->nt), sd = static_cast<size_t>(s->shape.sd);
    const size_t nck = static_cast<size_t>(max_steps / segment + 1);
    const size_t b_dt = align256(static_cast<size_t>(max_steps) * nt * 8), b_cx = align256(nck * sd * nt * 8);
    const size_t b_ct = align256(nck * nt * 8), b_n = align256(nt * 4);
    const size_t need = b_dt + b_cx + b_ct + b_n;
    if (need > MPGOS_STATIC_TAPE_BYTES)
        return fail(MPGOS_ERR_ARGUMENT,
                    "static tape: %zu bytes needed for %zu instances x %d steps (checkpoint every %d), only %zu "
                    "available (MPGOS_STATIC_TAPE_BYTES); use mpgos_pt_solve_record",
                    need, nt, max_steps, segment, static_cast<size_t>(MPGOS_STATIC_TAPE_BYTES));
    MPGOS_CUDA(cudaSetDevice(s->device));
    unsigned char* base = nullptr;
    if ((rc = static_tape_base(s->device, &base))) return rc;
    mpgos_pt_tape t{};
    t.segment = segment;
    t.max_steps = max_steps;
    t.dt = reinterpret_cast<double*>(base);
    t.ckpt_x = reinterpret_cast<double*>(base + b_dt);
    t.ckpt_t = reinterpret_cast<double*>(base + b_dt + b_cx);
    t.n_steps = reinterpret_cast<int32_t*>(base + b_dt + b_cx + b_ct);
    s->static_tape = t;
    s->use_static_tape = true;
    // step counts of instances this launch does not integrate read as zero
    MPGOS_CUDA(cudaMemsetAsync(t.n_steps, 0, nt * 4, s->stream));
    if (s->n_active <= 0) return MPGOS_OK;
    const int32_t m = effective_mode(s, s->mode) & (MPGOS_MODE_FAST_CONTROL | MPGOS_MODE_PERSISTENT | MPGOS_MODE_DF_STAGE |
                                                   MPGOS_MODE_SPLIT);
    int grid = 0;
    if ((rc = grid_for(s, m, s->block, &grid))) return rc;
    if (m & MPGOS_MODE_PERSISTENT) MPGOS_CUDA(cudaMemsetAsync(s->d_work, 0, sizeof(uint32_t), s->stream));
    mpgos_pt_launch L;
    fill_launch(s, L, m);
    rc = s->k->launch_record(&L, &s->static_tape, grid, s->block, dynamic_smem(s), s->stream);
    if (rc != 0) return fail(MPGOS_ERR_CUDA, "recording launch failed: %s", cudaGetErrorString((cudaError_t)rc));
    return MPGOS_OK;
}
