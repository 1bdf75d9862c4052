// Host runtime of the coupled per-block solver: the mpgos_cb_* functions of
// mpgos.h, playing the role of the reference's coupled ProblemSolver
// (SourceCodes/CoupledSystems_PerBlock_Interface.cuh:135-248, :350-1990):
// pinned host + device buffers, stream and event, options, synchronisation
// and the launch of a coupled-system plugin's kernels (one warp per system).
#include "mpgos.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#define MPGOS_EXPORT extern "C" __attribute__((visibility("default")))

// Shared with runtime.cpp: thread-local last error.
extern "C" const char* mpgos_last_error(void);
namespace mpgos_runtime {
int set_error(int code, const char* msg);
}

namespace {

int fail(int code, const char* fmt, ...)
{
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    return mpgos_runtime::set_error(code, buf);
}

#define CB_CUDA(call)                                                                                      \
    do {                                                                                                   \
        cudaError_t e_ = (call);                                                                           \
        if (e_ != cudaSuccess)                                                                             \
            return fail(MPGOS_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                        __LINE__);                                                                         \
    } while (0)

struct Buf {
    void* host = nullptr;
    void* device = nullptr;
    int64_t count = 0;
    size_t elem = 0;
    size_t bytes() const { return static_cast<size_t>(count) * elem; }
};

constexpr int kVars = 40;

}  // namespace

struct mpgos_cb_solver {
    const mpgos_cb_kernels* k = nullptr;
    mpgos_cb_shape sh{};
    int64_t ns = 0;
    int32_t ndo = 0;
    int device = 0, sm_count = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t sync_event = nullptr, t0 = nullptr, t1 = nullptr;
    Buf var[kVars];
    void *d_rtol = nullptr, *d_atol = nullptr, *d_etol = nullptr;
    int32_t* d_edir = nullptr;
    uint32_t* d_work = nullptr;
    std::vector<double> rtol, atol, etol;
    std::vector<int32_t> edir;
    // options (CoupledSystems_PerBlock_Interface.cuh:613-635)
    int64_t n_active = 0;
    double initial_dt = 1e-2, max_dt = 1e6, min_dt = 1e-12, grow = 5.0, shrink = 0.1, dense_min_dt = 0.0;
    int32_t dense_freq = 1, shared_global = 1, shared_coupling = 1, mode = 0, warps = 4;
    int64_t max_attempts = 10000000;
    std::vector<void*> ckpt;
    mpgos_pt_tape tape{};  // discrete-adjoint tape (mpgos_cb_solve_record)
    void* d_cmat_df = nullptr;  // DF_STAGE: double-float copy of matrices too large for shared memory
};

namespace {
// FP64 coupling matrices to double-float pairs (hi = the nearest float, lo =
// the nearest float to the remainder), converted on the solver's stream
// before every DF_STAGE launch that reads them from global memory.
__global__ void matrix_to_double_float(const double* in, float2* out, long long n)
{
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const double d = in[i];
        const float hi = static_cast<float>(d);
        out[i] = make_float2(hi, static_cast<float>(d - static_cast<double>(hi)));
    }
}
}  // namespace

namespace {

size_t prec(const mpgos_cb_solver* s) { return static_cast<size_t>(s->sh.precision_bytes); }

int check(const mpgos_cb_solver* s) { return s ? MPGOS_OK : fail(MPGOS_ERR_ARGUMENT, "null coupled solver handle"); }

bool valid_var(int32_t v) { return (v >= MPGOS_CB_TIME_DOMAIN && v <= MPGOS_CB_DENSE_STATE && v != MPGOS_CB_DENSE_OUTPUT) || (v >= MPGOS_CB_STATUS && v <= MPGOS_CB_REJECTED_STEPS); }

int push_options(mpgos_cb_solver* s)
{
    const size_t p = prec(s);
    auto put = [&](void* dst, const std::vector<double>& v) -> int {
        if (v.empty()) return MPGOS_OK;
        std::vector<unsigned char> tmp(v.size() * p);
        for (size_t i = 0; i < v.size(); i++) {
            if (p == 8) {
                std::memcpy(&tmp[i * p], &v[i], 8);
            } else {
                const float f = static_cast<float>(v[i]);
                std::memcpy(&tmp[i * p], &f, 4);
            }
        }
        CB_CUDA(cudaMemcpy(dst, tmp.data(), tmp.size(), cudaMemcpyHostToDevice));
        return MPGOS_OK;
    };
    CB_CUDA(cudaSetDevice(s->device));
    CB_CUDA(cudaStreamSynchronize(s->stream));
    int rc;
    if ((rc = put(s->d_rtol, s->rtol)) || (rc = put(s->d_atol, s->atol)) || (rc = put(s->d_etol, s->etol))) return rc;
    if (!s->edir.empty())
        CB_CUDA(cudaMemcpy(s->d_edir, s->edir.data(), s->edir.size() * 4, cudaMemcpyHostToDevice));
    return MPGOS_OK;
}

std::vector<int32_t> expand(int32_t v)
{
    if (v == MPGOS_CB_ALL)
        return {MPGOS_CB_TIME_DOMAIN, MPGOS_CB_ACTUAL_TIME, MPGOS_CB_ACTUAL_STATE, MPGOS_CB_UNIT_PARAMETERS,
                MPGOS_CB_SYSTEM_PARAMETERS, MPGOS_CB_GLOBAL_PARAMETERS, MPGOS_CB_INTEGER_GLOBAL_PARAMETERS,
                MPGOS_CB_UNIT_ACCESSORIES, MPGOS_CB_INTEGER_UNIT_ACCESSORIES, MPGOS_CB_SYSTEM_ACCESSORIES,
                MPGOS_CB_INTEGER_SYSTEM_ACCESSORIES, MPGOS_CB_COUPLING_MATRIX, MPGOS_CB_COUPLING_STRENGTH,
                MPGOS_CB_COUPLING_INDEX, MPGOS_CB_DENSE_INDEX, MPGOS_CB_DENSE_TIME, MPGOS_CB_DENSE_STATE};
    if (v == MPGOS_CB_DENSE_OUTPUT) return {MPGOS_CB_DENSE_INDEX, MPGOS_CB_DENSE_TIME, MPGOS_CB_DENSE_STATE};
    if (valid_var(v)) return {v};
    return {};
}

const int32_t kMutable[] = {MPGOS_CB_TIME_DOMAIN, MPGOS_CB_ACTUAL_TIME, MPGOS_CB_ACTUAL_STATE,
                            MPGOS_CB_UNIT_ACCESSORIES, MPGOS_CB_INTEGER_UNIT_ACCESSORIES, MPGOS_CB_SYSTEM_ACCESSORIES,
                            MPGOS_CB_INTEGER_SYSTEM_ACCESSORIES, MPGOS_CB_DENSE_INDEX, MPGOS_CB_DENSE_TIME,
                            MPGOS_CB_DENSE_STATE};

}  // namespace

MPGOS_EXPORT int mpgos_cb_destroy(mpgos_cb_solver* s)
{
    if (!s) return MPGOS_OK;
    cudaSetDevice(s->device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    for (Buf& b : s->var) {
        if (b.host) cudaFreeHost(b.host);
        if (b.device) cudaFree(b.device);
    }
    for (void* p : {s->d_rtol, s->d_atol, s->d_etol, static_cast<void*>(s->d_edir), static_cast<void*>(s->d_work),
                    s->d_cmat_df})
        if (p) cudaFree(p);
    for (void* p : s->ckpt)
        if (p) cudaFree(p);
    for (void* p : {static_cast<void*>(s->tape.dt), static_cast<void*>(s->tape.ckpt_x),
                    static_cast<void*>(s->tape.ckpt_t), static_cast<void*>(s->tape.n_steps)})
        if (p) cudaFree(p);
    if (s->t0) cudaEventDestroy(s->t0);
    if (s->t1) cudaEventDestroy(s->t1);
    if (s->sync_event) cudaEventDestroy(s->sync_event);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return MPGOS_OK;
}

MPGOS_EXPORT int mpgos_cb_create(const mpgos_cb_kernels* kernels, int64_t ns, int32_t ndo, int device, mpgos_cb_solver** out)
{
    mpgos_runtime::set_error(MPGOS_OK, "");
    if (!out) return fail(MPGOS_ERR_ARGUMENT, "null output handle");
    *out = nullptr;
    if (!kernels) return fail(MPGOS_ERR_ARGUMENT, "null coupled kernel table");
    if (kernels->abi_version != MPGOS_ABI_VERSION) return fail(MPGOS_ERR_SHAPE, "coupled kernel table ABI mismatch");
    const mpgos_cb_shape& sh = kernels->shape;
    if (sh.ups < 1 || sh.ud < 1 || (sh.precision_bytes != 4 && sh.precision_bytes != 8))
        return fail(MPGOS_ERR_SHAPE, "invalid coupled shape");
    if (ns < 1 || ns * sh.ups > 0x7FFFFFFF) return fail(MPGOS_ERR_ARGUMENT, "number of systems %lld out of range", (long long)ns);
    if (ndo < 0) return fail(MPGOS_ERR_ARGUMENT, "negative number of dense-output points");
    mpgos_cb_solver* s = new mpgos_cb_solver();
    s->k = kernels;
    s->sh = sh;
    s->ns = ns;
    s->ndo = ndo;
    s->device = device;
    s->n_active = ns;
    auto bail = [&](int rc) {
        mpgos_cb_destroy(s);
        return rc;
    };
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return bail(fail(MPGOS_ERR_CUDA, "cudaSetDevice(%d): %s", device, cudaGetErrorString(e)));
    if ((e = cudaDeviceGetAttribute(&s->sm_count, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&s->sync_event, cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaEventCreate(&s->t0)) != cudaSuccess || (e = cudaEventCreate(&s->t1)) != cudaSuccess)
        return bail(fail(MPGOS_ERR_CUDA, "stream/event creation: %s", cudaGetErrorString(e)));
    const int64_t nu = ns * sh.ups, p = sh.precision_bytes;
    const int64_t rows[][3] = {
        {MPGOS_CB_TIME_DOMAIN, 2 * ns, p}, {MPGOS_CB_ACTUAL_TIME, ns, p}, {MPGOS_CB_ACTUAL_STATE, sh.ud * nu, p},
        {MPGOS_CB_UNIT_PARAMETERS, sh.nup * nu, p}, {MPGOS_CB_SYSTEM_PARAMETERS, sh.nsp * ns, p},
        {MPGOS_CB_GLOBAL_PARAMETERS, sh.ngp, p}, {MPGOS_CB_INTEGER_GLOBAL_PARAMETERS, sh.nigp, 4},
        {MPGOS_CB_UNIT_ACCESSORIES, sh.nua * nu, p}, {MPGOS_CB_INTEGER_UNIT_ACCESSORIES, sh.niua * nu, 4},
        {MPGOS_CB_SYSTEM_ACCESSORIES, sh.nsa * ns, p}, {MPGOS_CB_INTEGER_SYSTEM_ACCESSORIES, sh.nisa * ns, 4},
        {MPGOS_CB_COUPLING_MATRIX, static_cast<int64_t>(sh.nc) * sh.matrix_entries, p},
        {MPGOS_CB_COUPLING_STRENGTH, sh.nc * ns, p}, {MPGOS_CB_COUPLING_INDEX, sh.nc, 4},
        {MPGOS_CB_DENSE_INDEX, ns, 4}, {MPGOS_CB_DENSE_TIME, ndo * ns, p}, {MPGOS_CB_DENSE_STATE, ndo * sh.ud * nu, p},
        {MPGOS_CB_STATUS, ns, 4}, {MPGOS_CB_ACCEPTED_STEPS, ns, 4}, {MPGOS_CB_REJECTED_STEPS, ns, 4}};
    for (const auto& r : rows) {
        Buf& b = s->var[r[0]];
        b.count = r[1];
        b.elem = static_cast<size_t>(r[2]);
        const size_t bytes = std::max<size_t>(b.bytes(), 16);
        if (cudaMallocHost(&b.host, bytes) != cudaSuccess) return bail(fail(MPGOS_ERR_MEMORY, "pinned allocation of %zu bytes failed", bytes));
        std::memset(b.host, 0, bytes);
        if (cudaMalloc(&b.device, bytes) != cudaSuccess) return bail(fail(MPGOS_ERR_MEMORY, "device allocation of %zu bytes failed", bytes));
        if (cudaMemset(b.device, 0, bytes) != cudaSuccess) return bail(fail(MPGOS_ERR_CUDA, "device memset failed"));
    }
    // defaults: coupling strength 1, coupling index 0 (the user sets them)
    if (p == 8) {
        double* cs = static_cast<double*>(s->var[MPGOS_CB_COUPLING_STRENGTH].host);
        for (int64_t i = 0; i < sh.nc * ns; i++) cs[i] = 1.0;
    } else {
        float* cs = static_cast<float*>(s->var[MPGOS_CB_COUPLING_STRENGTH].host);
        for (int64_t i = 0; i < sh.nc * ns; i++) cs[i] = 1.0f;
    }
    auto dalloc = [&](void** q, size_t bytes) {
        bytes = std::max<size_t>(bytes, 16);
        return cudaMalloc(q, bytes) == cudaSuccess && cudaMemset(*q, 0, bytes) == cudaSuccess;
    };
    if (!dalloc(&s->d_rtol, p * sh.ud) || !dalloc(&s->d_atol, p * sh.ud) || !dalloc(&s->d_etol, p * sh.ne) ||
        !dalloc(reinterpret_cast<void**>(&s->d_edir), 4 * sh.ne) || !dalloc(reinterpret_cast<void**>(&s->d_work), 4))
        return bail(fail(MPGOS_ERR_MEMORY, "device allocation of option arrays failed"));
    s->rtol.assign(sh.ud, 1e-8);
    s->atol.assign(sh.ud, 1e-8);
    s->etol.assign(sh.ne, 1e-6);
    s->edir.assign(sh.ne, 0);
    int rc = push_options(s);
    if (rc) return bail(rc);
    *out = s;
    return MPGOS_OK;
}

MPGOS_EXPORT int mpgos_cb_get_shape(const mpgos_cb_solver* s, mpgos_cb_shape* shape, int64_t* ns, int32_t* ndo)
{
    int rc = check(s);
    if (rc) return rc;
    if (shape) *shape = s->sh;
    if (ns) *ns = s->ns;
    if (ndo) *ndo = s->ndo;
    return MPGOS_OK;
}

MPGOS_EXPORT int mpgos_cb_set_option(mpgos_cb_solver* s, int32_t option, int32_t index, double value)
{
    int rc = check(s);
    if (rc) return rc;
    auto positive = [&](const char* n) { return (value > 0.0 && std::isfinite(value)) ? MPGOS_OK : fail(MPGOS_ERR_ARGUMENT, "SolverOption %s: %g must be positive", n, value); };
    auto idx = [&](const char* n, int32_t lim) { return (index >= 0 && index < lim) ? MPGOS_OK : fail(MPGOS_ERR_ARGUMENT, "SolverOption %s: index %d outside 0..%d", n, index, lim - 1); };
    switch (option) {
        case MPGOS_CB_INITIAL_TIME_STEP: if ((rc = positive("InitialTimeStep"))) return rc; s->initial_dt = value; break;
        case MPGOS_CB_ACTIVE_SYSTEMS: {
            const int64_t n = static_cast<int64_t>(value);
            if (n < 0 || n > s->ns || n != value) return fail(MPGOS_ERR_ARGUMENT, "ActiveSystems %g outside 0..%lld", value, (long long)s->ns);
            s->n_active = n;
            break;
        }
        case MPGOS_CB_MAXIMUM_TIME_STEP: if ((rc = positive("MaximumTimeStep"))) return rc; s->max_dt = value; break;
        case MPGOS_CB_MINIMUM_TIME_STEP: if ((rc = positive("MinimumTimeStep"))) return rc; s->min_dt = value; break;
        case MPGOS_CB_TIME_STEP_GROW_LIMIT: if ((rc = positive("TimeStepGrowLimit"))) return rc; s->grow = value; break;
        case MPGOS_CB_TIME_STEP_SHRINK_LIMIT: if ((rc = positive("TimeStepShrinkLimit"))) return rc; s->shrink = value; break;
        case MPGOS_CB_DENSE_OUTPUT_MINIMUM_TIME_STEP:
            if (!(value >= 0.0)) return fail(MPGOS_ERR_ARGUMENT, "DenseOutputMinimumTimeStep must be >= 0");
            s->dense_min_dt = value;
            break;
        case MPGOS_CB_DENSE_OUTPUT_SAVE_FREQUENCY:
            if (value < 1 || value != static_cast<int>(value)) return fail(MPGOS_ERR_ARGUMENT, "DenseOutputSaveFrequency must be >= 1");
            s->dense_freq = static_cast<int32_t>(value);
            break;
        case MPGOS_CB_SHARED_GLOBAL_VARIABLES: s->shared_global = value != 0.0; break;
        case MPGOS_CB_SHARED_COUPLING_MATRICES: s->shared_coupling = value != 0.0; break;
        case MPGOS_CB_RELATIVE_TOLERANCE:
        case MPGOS_CB_ABSOLUTE_TOLERANCE:
            if ((rc = idx("Tolerance", s->sh.ud))) return rc;
            if (!(value >= 0.0) || !std::isfinite(value)) return fail(MPGOS_ERR_ARGUMENT, "tolerance must be finite and >= 0");
            (option == MPGOS_CB_RELATIVE_TOLERANCE ? s->rtol : s->atol)[index] = value;
            return push_options(s);
        case MPGOS_CB_EVENT_TOLERANCE:
            if ((rc = idx("EventTolerance", s->sh.ne))) return rc;
            s->etol[index] = value;
            return push_options(s);
        case MPGOS_CB_EVENT_DIRECTION:
            if ((rc = idx("EventDirection", s->sh.ne))) return rc;
            s->edir[index] = static_cast<int32_t>(value);
            return push_options(s);
        case MPGOS_CB_KERNEL_MODE:
            if (value < 0 || value != static_cast<int>(value) ||
                (static_cast<int32_t>(value) &
                 ~(MPGOS_MODE_PERSISTENT | MPGOS_MODE_DF_STAGE | MPGOS_MODE_SPLIT | MPGOS_MODE_FAST_CONTROL)))
                return fail(MPGOS_ERR_ARGUMENT, "coupled kernel mode %g: only PERSISTENT, DF_STAGE and SPLIT apply",
                            value);
            if ((static_cast<int32_t>(value) & MPGOS_MODE_DF_STAGE) && (static_cast<int32_t>(value) & MPGOS_MODE_SPLIT))
                return fail(MPGOS_ERR_ARGUMENT, "coupled kernel mode %g: DF_STAGE and SPLIT exclude each other", value);
            if ((static_cast<int32_t>(value) & (MPGOS_MODE_DF_STAGE | MPGOS_MODE_SPLIT)) && s->sh.precision_bytes != 8)
                return fail(MPGOS_ERR_UNSUPPORTED, "DF_STAGE and SPLIT need a double-precision coupled table");
            s->mode = static_cast<int32_t>(value) & (MPGOS_MODE_PERSISTENT | MPGOS_MODE_DF_STAGE | MPGOS_MODE_SPLIT);
            break;
        case MPGOS_CB_MAXIMUM_ATTEMPTS:
            if (value < 1) return fail(MPGOS_ERR_ARGUMENT, "MaximumAttempts must be >= 1");
            s->max_attempts = static_cast<int64_t>(value);
            break;
        case MPGOS_CB_WARPS_PER_BLOCK:
            if (value < 1 || value > 8 || value != static_cast<int>(value)) return fail(MPGOS_ERR_ARGUMENT, "WarpsPerBlock %g outside 1..8", value);
            s->warps = static_cast<int32_t>(value);
            break;
        default: return fail(MPGOS_ERR_ARGUMENT, "unknown coupled solver option %d", option);
    }
    return MPGOS_OK;
}

MPGOS_EXPORT int mpgos_cb_host_buffer(mpgos_cb_solver* s, int32_t v, void** ptr, int64_t* count)
{
    int rc = check(s);
    if (rc) return rc;
    if (!valid_var(v)) return fail(MPGOS_ERR_ARGUMENT, "coupled variable %d has no single buffer", v);
    if (ptr) *ptr = s->var[v].host;
    if (count) *count = s->var[v].count;
    return MPGOS_OK;
}

MPGOS_EXPORT int mpgos_cb_device_buffer(mpgos_cb_solver* s, int32_t v, void** ptr, int64_t* count)
{
    int rc = check(s);
    if (rc) return rc;
    if (!valid_var(v)) return fail(MPGOS_ERR_ARGUMENT, "coupled variable %d has no single buffer", v);
    if (ptr) *ptr = s->var[v].device;
    if (count) *count = s->var[v].count;
    return MPGOS_OK;
}

MPGOS_EXPORT int mpgos_cb_sync_h2d(mpgos_cb_solver* s, int32_t v)
{
    int rc = check(s);
    if (rc) return rc;
    auto vs = expand(v);
    if (vs.empty()) return fail(MPGOS_ERR_ARGUMENT, "SynchroniseFromHostToDevice: variable %d not applicable", v);
    CB_CUDA(cudaSetDevice(s->device));
    for (int32_t x : vs)
        if (s->var[x].bytes()) CB_CUDA(cudaMemcpyAsync(s->var[x].device, s->var[x].host, s->var[x].bytes(), cudaMemcpyHostToDevice, s->stream));
    return MPGOS_OK;
}

MPGOS_EXPORT int mpgos_cb_sync_d2h(mpgos_cb_solver* s, int32_t v)
{
    int rc = check(s);
    if (rc) return rc;
    auto vs = expand(v);
    if (vs.empty()) return fail(MPGOS_ERR_ARGUMENT, "SynchroniseFromDeviceToHost: variable %d not applicable", v);
    CB_CUDA(cudaSetDevice(s->device));
    for (int32_t x : vs)
        if (s->var[x].bytes()) CB_CUDA(cudaMemcpyAsync(s->var[x].host, s->var[x].device, s->var[x].bytes(), cudaMemcpyDeviceToHost, s->stream));
    return MPGOS_OK;
}

namespace {
// Launch configuration and arguments of one Solve() (record = the recording
// forward launch of the discrete adjoint, which uses the FP64 kernels).
int prepare_launch(mpgos_cb_solver* s, bool record, mpgos_cb_launch& L, int64_t& grid_out, int& block_out,
                   size_t& smem_out);
}  // namespace

MPGOS_EXPORT int mpgos_cb_solve(mpgos_cb_solver* s)
{
    int rc = check(s);
    if (rc) return rc;
    if (s->n_active <= 0) return MPGOS_OK;
    CB_CUDA(cudaSetDevice(s->device));
    mpgos_cb_launch L;
    int64_t grid = 0;
    int block = 0;
    size_t smem = 0;
    if ((rc = prepare_launch(s, false, L, grid, block, smem))) return rc;
    int e = s->k->launch(&L, static_cast<int>(grid), block, smem, s->stream);
    if (e != 0) return fail(MPGOS_ERR_CUDA, "coupled kernel launch failed: %s", cudaGetErrorString((cudaError_t)e));
    return MPGOS_OK;
}

namespace {
int prepare_launch(mpgos_cb_solver* s, bool record, mpgos_cb_launch& L, int64_t& grid_out, int& block_out,
                   size_t& smem_out)
{
    const int32_t mode =
        record ? (s->mode & (MPGOS_MODE_PERSISTENT | MPGOS_MODE_DF_STAGE | MPGOS_MODE_SPLIT)) : s->mode;
    const int block = 32 * s->warps;
    // the double-float kernels (DF_STAGE, and SPLIT for its right-hand side)
    // stage double-float copies of the global parameters and matrices
    const bool df = (mode & (MPGOS_MODE_DF_STAGE | MPGOS_MODE_SPLIT)) != 0;
    const long long n_matrix = static_cast<long long>(s->sh.nc) * s->sh.matrix_entries;
    // DF_STAGE: matrices in shared memory exactly when the kernel's
    // compile-time rule says so (MPGOS_CB_DF_SHARED_MATRIX_BYTES)
    const int df_sc = n_matrix * 8 <= static_cast<long long>(MPGOS_CB_DF_SHARED_MATRIX_BYTES) ? 1 : 0;
    int sg = df ? 1 : s->shared_global, sc = df ? df_sc : s->shared_coupling;
    size_t smem = s->k->dynamic_smem(s->warps, sg, sc);
    const void* cmat_df = nullptr;
    if (!df && smem > 200 * 1024 && sc) {  // coupling matrix too large for shared memory: read it from global
        sc = 0;
        smem = s->k->dynamic_smem(s->warps, sg, sc);
    }
    if (df && !sc) {
        // the double-float kernels read a double-float copy, refreshed before every launch
        if (s->d_cmat_df == nullptr && cudaMalloc(&s->d_cmat_df, static_cast<size_t>(n_matrix) * 8) != cudaSuccess) {
            s->d_cmat_df = nullptr;
            return fail(MPGOS_ERR_MEMORY, "double-float coupling matrix copy (%lld entries) allocation failed",
                        n_matrix);
        }
        const int blocks = static_cast<int>(std::min<long long>((n_matrix + 255) / 256, 4096));
        matrix_to_double_float<<<blocks, 256, 0, s->stream>>>(
            static_cast<const double*>(s->var[MPGOS_CB_COUPLING_MATRIX].device), static_cast<float2*>(s->d_cmat_df),
            n_matrix);
        CB_CUDA(cudaGetLastError());
        cmat_df = s->d_cmat_df;
    }
    if (smem > 227 * 1024)
        return fail(MPGOS_ERR_ARGUMENT, "coupled launch needs %zu bytes of shared memory; use fewer warps per block",
                    smem);
    int64_t grid = (s->n_active + s->warps - 1) / s->warps;
    if (mode & MPGOS_MODE_PERSISTENT) {
        int per_sm = 0;
        int e = s->k->occupancy(mode, block, smem, &per_sm);
        if (e != 0) return fail(MPGOS_ERR_CUDA, "coupled occupancy query: %s", cudaGetErrorString((cudaError_t)e));
        grid = std::min<int64_t>(grid, static_cast<int64_t>(std::max(per_sm, 1)) * s->sm_count);
        CB_CUDA(cudaMemsetAsync(s->d_work, 0, 4, s->stream));
    }
    std::memset(&L, 0, sizeof(L));
    L.ns = s->ns;
    L.n_active = s->n_active;
    L.ndo = s->ndo;
    L.mode = mode;
    L.shared_global = sg;
    L.shared_coupling = sc;
    L.dense_save_frequency = s->dense_freq;
    L.max_attempts = s->max_attempts;
    L.initial_dt = s->initial_dt;
    L.max_dt = s->max_dt;
    L.min_dt = s->min_dt;
    L.grow_limit = s->grow;
    L.shrink_limit = s->shrink;
    L.dense_min_dt = s->dense_min_dt;
    auto d = [&](int32_t v) { return s->var[v].device; };
    L.time_domain = d(MPGOS_CB_TIME_DOMAIN);
    L.actual_time = d(MPGOS_CB_ACTUAL_TIME);
    L.system_parameters = d(MPGOS_CB_SYSTEM_PARAMETERS);
    L.system_accessories = d(MPGOS_CB_SYSTEM_ACCESSORIES);
    L.integer_system_accessories = static_cast<int32_t*>(d(MPGOS_CB_INTEGER_SYSTEM_ACCESSORIES));
    L.coupling_strength = d(MPGOS_CB_COUPLING_STRENGTH);
    L.dense_index = static_cast<int32_t*>(d(MPGOS_CB_DENSE_INDEX));
    L.dense_time = d(MPGOS_CB_DENSE_TIME);
    L.actual_state = d(MPGOS_CB_ACTUAL_STATE);
    L.unit_parameters = d(MPGOS_CB_UNIT_PARAMETERS);
    L.unit_accessories = d(MPGOS_CB_UNIT_ACCESSORIES);
    L.integer_unit_accessories = static_cast<int32_t*>(d(MPGOS_CB_INTEGER_UNIT_ACCESSORIES));
    L.dense_state = d(MPGOS_CB_DENSE_STATE);
    L.global_parameters = d(MPGOS_CB_GLOBAL_PARAMETERS);
    L.integer_global_parameters = static_cast<const int32_t*>(d(MPGOS_CB_INTEGER_GLOBAL_PARAMETERS));
    L.coupling_matrix = d(MPGOS_CB_COUPLING_MATRIX);
    L.coupling_matrix_df = cmat_df;
    L.coupling_index = static_cast<const int32_t*>(d(MPGOS_CB_COUPLING_INDEX));
    L.relative_tolerance = s->d_rtol;
    L.absolute_tolerance = s->d_atol;
    L.event_tolerance = s->d_etol;
    L.event_direction = s->d_edir;
    L.status = static_cast<int32_t*>(d(MPGOS_CB_STATUS));
    L.accepted_steps = static_cast<int32_t*>(d(MPGOS_CB_ACCEPTED_STEPS));
    L.rejected_steps = static_cast<int32_t*>(d(MPGOS_CB_REJECTED_STEPS));
    L.work_counter = s->d_work;
    // coupling indices must address a unit-state component
    const int32_t* ci = static_cast<const int32_t*>(s->var[MPGOS_CB_COUPLING_INDEX].host);
    for (int i = 0; i < s->sh.nc; i++)
        if (ci[i] < 0 || ci[i] >= s->sh.ud) return fail(MPGOS_ERR_ARGUMENT, "CouplingIndex[%d] = %d outside 0..%d", i, ci[i], s->sh.ud - 1);
    grid_out = grid;
    block_out = block;
    smem_out = smem;
    return MPGOS_OK;
}
}  // namespace

MPGOS_EXPORT int mpgos_cb_solve_record(mpgos_cb_solver* s, int32_t max_steps, int32_t segment)
{
    int rc = check(s);
    if (rc) return rc;
    if (s->k->launch_record == nullptr || s->sh.precision_bytes != 8)
        return fail(MPGOS_ERR_UNSUPPORTED, "coupled system %s has no adjoint kernels (FP64 only)", s->k->name);
    if (max_steps < 1 || segment < 1 || segment > 64)
        return fail(MPGOS_ERR_ARGUMENT, "tape: max_steps %d must be >= 1 and segment %d within 1..64", max_steps, segment);
    CB_CUDA(cudaSetDevice(s->device));
    const size_t ns = static_cast<size_t>(s->ns), nu = ns * static_cast<size_t>(s->sh.ups);
    const size_t ud = static_cast<size_t>(s->sh.ud), nck = static_cast<size_t>(max_steps / segment + 1);
    if (s->tape.max_steps != max_steps || s->tape.segment != segment || s->tape.dt == nullptr) {
        CB_CUDA(cudaStreamSynchronize(s->stream));
        for (void* p : {static_cast<void*>(s->tape.dt), static_cast<void*>(s->tape.ckpt_x),
                        static_cast<void*>(s->tape.ckpt_t), static_cast<void*>(s->tape.n_steps)})
            if (p) cudaFree(p);
        s->tape = mpgos_pt_tape{};
        const size_t b_dt = static_cast<size_t>(max_steps) * ns * 8, b_cx = nck * ud * nu * 8, b_ct = nck * ns * 8;
        if (cudaMalloc(reinterpret_cast<void**>(&s->tape.dt), b_dt) != cudaSuccess ||
            cudaMalloc(reinterpret_cast<void**>(&s->tape.ckpt_x), b_cx) != cudaSuccess ||
            cudaMalloc(reinterpret_cast<void**>(&s->tape.ckpt_t), b_ct) != cudaSuccess ||
            cudaMalloc(reinterpret_cast<void**>(&s->tape.n_steps), ns * 4) != cudaSuccess) {
            s->tape.max_steps = 0;
            return fail(MPGOS_ERR_MEMORY, "coupled adjoint tape allocation (%zu bytes) failed", b_dt + b_cx + b_ct + ns * 4);
        }
        s->tape.max_steps = max_steps;
        s->tape.segment = segment;
    }
    if (s->n_active <= 0) return MPGOS_OK;
    mpgos_cb_launch L;
    int64_t grid = 0;
    int block = 0;
    size_t smem = 0;
    if ((rc = prepare_launch(s, true, L, grid, block, smem))) return rc;
    int e = s->k->launch_record(&L, &s->tape, static_cast<int>(grid), block, smem, s->stream);
    if (e != 0) return fail(MPGOS_ERR_CUDA, "coupled recording launch failed: %s", cudaGetErrorString((cudaError_t)e));
    return MPGOS_OK;
}

MPGOS_EXPORT int mpgos_cb_adjoint(mpgos_cb_solver* s, const double* dLdxT, double* dLdx0, double* dLdsp)
{
    int rc = check(s);
    if (rc) return rc;
    if (s->k->launch_adjoint == nullptr) return fail(MPGOS_ERR_UNSUPPORTED, "coupled system %s has no adjoint kernels", s->k->name);
    if (s->tape.dt == nullptr) return fail(MPGOS_ERR_ARGUMENT, "no recorded forward pass (call mpgos_cb_solve_record first)");
    if (dLdxT == nullptr || dLdx0 == nullptr || (dLdsp == nullptr && s->sh.nsp > 0))
        return fail(MPGOS_ERR_ARGUMENT, "null gradient buffer");
    if (s->n_active <= 0) return MPGOS_OK;
    CB_CUDA(cudaSetDevice(s->device));
    // the reverse pass computes in double-float when the solver's stages do
    const int32_t amode = (s->mode & (MPGOS_MODE_DF_STAGE | MPGOS_MODE_SPLIT)) ? MPGOS_MODE_DF_STAGE : 0;
    // warps (systems) per block: the most resident warps per SM, the smaller
    // block on ties (shared memory holds the coupling matrices once per block)
    int warps = 0, best = -1;
    for (int w : {1, 2, 4, 8}) {
        const size_t need = s->k->adjoint_smem(w, amode);
        if (need > 227 * 1024) break;
        int per_sm = 0;
        if (s->k->adjoint_occupancy == nullptr) {
            per_sm = w == 2 ? 1 : 0;  // no occupancy query: two warps per block
        } else {
            const int e = s->k->adjoint_occupancy(amode, 32 * w, need, &per_sm);
            if (e != 0) return fail(MPGOS_ERR_CUDA, "coupled adjoint occupancy query: %s", cudaGetErrorString((cudaError_t)e));
        }
        if (per_sm * w > best) {
            best = per_sm * w;
            warps = w;
        }
    }
    if (warps == 0 || best <= 0)
        return fail(MPGOS_ERR_ARGUMENT, "coupled adjoint needs %zu bytes of shared memory per system",
                    s->k->adjoint_smem(1, amode));
    const int block = 32 * warps;
    const size_t smem = s->k->adjoint_smem(warps, amode);
    const int64_t grid = (s->n_active + warps - 1) / warps;
    mpgos_cb_launch L;
    int64_t g = 0;
    int b = 0;
    size_t sm = 0;
    if ((rc = prepare_launch(s, true, L, g, b, sm))) return rc;
    int e = s->k->launch_adjoint(&L, &s->tape, dLdxT, dLdx0, dLdsp, static_cast<int>(grid), block, smem, s->stream);
    if (e != 0) return fail(MPGOS_ERR_CUDA, "coupled adjoint launch failed: %s", cudaGetErrorString((cudaError_t)e));
    return MPGOS_OK;
}

MPGOS_EXPORT int mpgos_cb_tape_info(const mpgos_cb_solver* s, mpgos_pt_tape* tape)
{
    int rc = check(s);
    if (rc) return rc;
    if (tape == nullptr) return fail(MPGOS_ERR_ARGUMENT, "null tape pointer");
    *tape = s->tape;
    return MPGOS_OK;
}

MPGOS_EXPORT int mpgos_cb_insert_sync_point(mpgos_cb_solver* s)
{
    int rc = check(s);
    if (rc) return rc;
    CB_CUDA(cudaSetDevice(s->device));
    CB_CUDA(cudaEventRecord(s->sync_event, s->stream));
    return MPGOS_OK;
}

MPGOS_EXPORT int mpgos_cb_sync_solver(mpgos_cb_solver* s)
{
    int rc = check(s);
    if (rc) return rc;
    CB_CUDA(cudaSetDevice(s->device));
    CB_CUDA(cudaEventSynchronize(s->sync_event));
    CB_CUDA(cudaGetLastError());
    return MPGOS_OK;
}

MPGOS_EXPORT int mpgos_cb_timer_start(mpgos_cb_solver* s)
{
    int rc = check(s);
    if (rc) return rc;
    CB_CUDA(cudaEventRecord(s->t0, s->stream));
    return MPGOS_OK;
}

MPGOS_EXPORT int mpgos_cb_timer_stop(mpgos_cb_solver* s, float* ms)
{
    int rc = check(s);
    if (rc) return rc;
    CB_CUDA(cudaEventRecord(s->t1, s->stream));
    CB_CUDA(cudaEventSynchronize(s->t1));
    float t = 0.f;
    CB_CUDA(cudaEventElapsedTime(&t, s->t0, s->t1));
    if (ms) *ms = t;
    return MPGOS_OK;
}

MPGOS_EXPORT int mpgos_cb_stream(mpgos_cb_solver* s, void** stream)
{
    int rc = check(s);
    if (rc) return rc;
    if (stream) *stream = s->stream;
    return MPGOS_OK;
}

MPGOS_EXPORT int mpgos_cb_checkpoint_save(mpgos_cb_solver* s)
{
    int rc = check(s);
    if (rc) return rc;
    CB_CUDA(cudaSetDevice(s->device));
    const size_t n = sizeof(kMutable) / sizeof(kMutable[0]);
    if (s->ckpt.empty()) {
        s->ckpt.assign(n, nullptr);
        for (size_t i = 0; i < n; i++)
            if (cudaMalloc(&s->ckpt[i], std::max<size_t>(s->var[kMutable[i]].bytes(), 16)) != cudaSuccess)
                return fail(MPGOS_ERR_MEMORY, "coupled checkpoint allocation failed");
    }
    for (size_t i = 0; i < n; i++)
        if (s->var[kMutable[i]].bytes())
            CB_CUDA(cudaMemcpyAsync(s->ckpt[i], s->var[kMutable[i]].device, s->var[kMutable[i]].bytes(), cudaMemcpyDeviceToDevice, s->stream));
    return MPGOS_OK;
}

MPGOS_EXPORT int mpgos_cb_checkpoint_restore(mpgos_cb_solver* s)
{
    int rc = check(s);
    if (rc) return rc;
    if (s->ckpt.empty()) return fail(MPGOS_ERR_ARGUMENT, "no coupled checkpoint saved");
    CB_CUDA(cudaSetDevice(s->device));
    const size_t n = sizeof(kMutable) / sizeof(kMutable[0]);
    for (size_t i = 0; i < n; i++)
        if (s->var[kMutable[i]].bytes())
            CB_CUDA(cudaMemcpyAsync(s->var[kMutable[i]].device, s->ckpt[i], s->var[kMutable[i]].bytes(), cudaMemcpyDeviceToDevice, s->stream));
    return MPGOS_OK;
}
