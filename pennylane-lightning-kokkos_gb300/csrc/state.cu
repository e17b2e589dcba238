// state.cu — library plumbing and state lifecycle of the C ABI.
//
// Replaces StateVectorKokkos's constructor / init / data movers
// (simulator/StateVectorKokkos.hpp:140-574, 1596-1636) and the Kokkos
// runtime configuration queries (util/GetConfigInfo.hpp).
#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "plk_internal.cuh"

namespace plk {

// ---------------------------------------------------------------- errors --
namespace {
thread_local std::string g_error;
}
void set_error(const std::string &msg) { g_error = msg; }
const std::string &last_error() { return g_error; }

// --------------------------------------------------------------- devices --
namespace {
std::mutex g_dev_mutex;
DeviceCtx g_dev[64];
bool g_dev_init[64] = {false};
} // namespace

int device_ctx(int device, DeviceCtx **out) {
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        PLK_FAIL(PLK_ERR_NO_DEVICE, "no CUDA device available");
    }
    if (device < 0 || device >= count || device >= 64)
        PLK_FAIL(PLK_ERR_INVALID_ARG, "device id " + std::to_string(device) + " out of range");
    std::lock_guard<std::mutex> lk(g_dev_mutex);
    if (!g_dev_init[device]) {
        PLK_CUDA(cudaSetDevice(device));
        cudaDeviceProp p;
        PLK_CUDA(cudaGetDeviceProperties(&p, device));
        g_dev[device].sm_count = p.multiProcessorCount;
        g_dev[device].max_threads_per_sm = p.maxThreadsPerMultiProcessor;
        PLK_CUDA(cudaStreamCreateWithFlags(&g_dev[device].stream, cudaStreamNonBlocking));
        // Freed state buffers stay mapped in the pool (up to the threshold),
        // so creating a state of a size seen before costs no page mapping and
        // destroying one no device-wide synchronisation.
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = device;
        PLK_CUDA(cudaMemPoolCreate(&g_dev[device].pool, &props));
        uint64_t keep = std::min<uint64_t>(16ull << 30, p.totalGlobalMem / 8);
        PLK_CUDA(cudaMemPoolSetAttribute(g_dev[device].pool, cudaMemPoolAttrReleaseThreshold, &keep));
        g_dev_init[device] = true;
    }
    *out = &g_dev[device];
    return PLK_OK;
}

int pool_alloc(int device, void **ptr, size_t bytes, cudaStream_t stream) {
    DeviceCtx *d = nullptr;
    PLK_TRY(device_ctx(device, &d));
    *ptr = nullptr;
    cudaError_t e = cudaMallocFromPoolAsync(ptr, bytes, d->pool, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        if (*ptr) cudaFreeAsync(*ptr, stream);
        *ptr = nullptr;
        PLK_FAIL(e == cudaErrorMemoryAllocation ? PLK_ERR_OUT_OF_MEMORY : PLK_ERR_CUDA,
                 "allocation of " + std::to_string(bytes) + " bytes failed: " + cudaGetErrorString(e));
    }
    return PLK_OK;
}

void pool_free(void *ptr, cudaStream_t stream) {
    if (ptr) cudaFreeAsync(ptr, stream);
}

// small pinned host buffers for reduction results, recycled across states
namespace {
std::mutex g_pinned_mutex;
std::vector<double *> g_pinned_free;
} // namespace

static int pinned_get(double **out) {
    {
        std::lock_guard<std::mutex> lk(g_pinned_mutex);
        if (!g_pinned_free.empty()) {
            *out = g_pinned_free.back();
            g_pinned_free.pop_back();
            return PLK_OK;
        }
    }
    PLK_CUDA(cudaMallocHost((void **)out, sizeof(double) * kMaxRedValues));
    return PLK_OK;
}

static void pinned_put(double *p) {
    if (!p) return;
    std::lock_guard<std::mutex> lk(g_pinned_mutex);
    g_pinned_free.push_back(p);
}

// complex128 arithmetic: 1 = double-float on the FP32 pipe (default), 0 =
// native FP64.  The environment sets the initial mode; plk_set_c128_arithmetic
// changes it for the calls that follow (each launch reads it once).
static std::atomic<int> g_c128_df{[] {
    const char *v = std::getenv("PLK_C128_ARITH");
    return (v && std::string(v) == "fp64") ? 0 : 1;
}()};

bool c128_use_df() { return g_c128_df.load(std::memory_order_relaxed) != 0; }

int device_sm_count(int device) {
    DeviceCtx *d = nullptr;
    if (device_ctx(device, &d) != PLK_OK) return 1;
    return d->sm_count;
}

int red_grid(const plk_state_s *s, uint64_t work_items) {
    DeviceCtx *d = nullptr;
    if (device_ctx(s->device, &d) != PLK_OK) return 1;
    uint64_t want = (work_items + kThreads - 1) / kThreads;
    uint64_t cap = (uint64_t)d->sm_count * 6;
    if (cap > (uint64_t)kMaxRedBlocks) cap = kMaxRedBlocks;
    if (want > cap) want = cap;
    return want < 1 ? 1 : (int)want;
}

Masks make_masks(const int *sorted, int count) {
    Masks mk{};
    for (int j = 0; j <= count; j++) {
        uint64_t lo = (j == 0) ? ~0ULL : (sorted[j - 1] + 1 >= 64 ? 0ULL : (~0ULL << (sorted[j - 1] + 1)));
        uint64_t hi = (j == count) ? ~0ULL : (sorted[j] == 0 ? 0ULL : (~0ULL >> (64 - sorted[j])));
        mk.m[j] = lo & hi;
    }
    for (int j = count + 1; j <= kMaxDenseWires; j++) mk.m[j] = 0;
    return mk;
}

int check_state(plk_state s) {
    if (!s || !s->data) PLK_FAIL(PLK_ERR_INVALID_ARG, "null or destroyed state");
    return PLK_OK;
}

int check_wires(plk_state s, const int64_t *wires, int nw) {
    if (nw < 0 || nw > s->nq) PLK_FAIL(PLK_ERR_INVALID_ARG, "wire count out of range");
    if (nw > 0 && !wires) PLK_FAIL(PLK_ERR_INVALID_ARG, "null wires");
    for (int i = 0; i < nw; i++) {
        if (wires[i] < 0 || wires[i] >= s->nq)
            PLK_FAIL(PLK_ERR_INVALID_ARG, "wire " + std::to_string(wires[i]) + " out of range for " +
                                              std::to_string(s->nq) + " qubits");
        for (int j = 0; j < i; j++)
            if (wires[i] == wires[j]) PLK_FAIL(PLK_ERR_INVALID_ARG, "repeated wire " + std::to_string(wires[i]));
    }
    return PLK_OK;
}

int order_after(plk_state s, plk_state other) {
    if (s->stream == other->stream) return PLK_OK;
    cudaEvent_t ev;
    PLK_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    PLK_CUDA(cudaEventRecord(ev, other->stream));
    PLK_CUDA(cudaStreamWaitEvent(s->stream, ev, 0));
    PLK_CUDA(cudaEventDestroy(ev));
    return PLK_OK;
}

// --------------------------------------------------------------- kernels --
template <class V> __global__ void k_fill_basis(V *__restrict__ a, uint64_t n, uint64_t index) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) {
        V v;
        v.x = (k == index) ? 1 : 0;
        v.y = 0;
        a[k] = v;
    }
}

template <class V>
__global__ void k_scatter(V *__restrict__ a, const uint64_t *__restrict__ idx, const V *__restrict__ val,
                          uint64_t count) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += stride)
        a[idx[k]] = val[k];
}

// y += a x; a real (the usual case: Hamiltonian coefficients) needs two FMAs
// per amplitude, which keeps complex128 within the FP64 pipe's budget at
// HBM speed.  Two amplitudes of x and y in flight per thread.
template <class V, class T, bool REAL>
__global__ void k_axpy(V *__restrict__ y, const V *__restrict__ x, T are, T aim, uint64_t n) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += 2 * stride) {
        const uint64_t k2 = k + stride;
        const bool two = k2 < n;
        const V x0 = x[k], y0 = y[k];
        V x1{}, y1{};
        if (two) {
            x1 = x[k2];
            y1 = y[k2];
        }
        V r0 = y0, r1 = y1;
        if (REAL) {
            r0.x = fma(are, x0.x, y0.x);
            r0.y = fma(are, x0.y, y0.y);
            r1.x = fma(are, x1.x, y1.x);
            r1.y = fma(are, x1.y, y1.y);
        } else {
            r0.x = fma(are, x0.x, fma(-aim, x0.y, y0.x));
            r0.y = fma(are, x0.y, fma(aim, x0.x, y0.y));
            r1.x = fma(are, x1.x, fma(-aim, x1.y, y1.x));
            r1.y = fma(are, x1.y, fma(aim, x1.x, y1.y));
        }
        y[k] = r0;
        if (two) y[k2] = r1;
    }
}

int elem_grid(plk_state s, uint64_t n) {
    DeviceCtx *d = nullptr;
    if (device_ctx(s->device, &d) != PLK_OK) return 1;
    uint64_t want = (n + kThreads - 1) / kThreads;
    uint64_t cap = (uint64_t)d->sm_count * (d->max_threads_per_sm / kThreads) * 4;
    if (want > cap) want = cap;
    return want < 1 ? 1 : (int)want;
}

int fill_basis(plk_state s, uint64_t index) {
    const int g = elem_grid(s, s->length);
    if (s->dtype == PLK_C64)
        k_fill_basis<float2><<<g, kThreads, 0, s->stream>>>((float2 *)s->data, s->length, index);
    else
        k_fill_basis<double2><<<g, kThreads, 0, s->stream>>>((double2 *)s->data, s->length, index);
    PLK_CHECK_LAUNCH();
    return PLK_OK;
}

} // namespace plk

using namespace plk;

// ------------------------------------------------------------------ C ABI --
extern "C" {

PLK_API const char *plk_last_error(void) { return plk::last_error().c_str(); }

PLK_API int plk_version(void) { return 1000; }

PLK_API int plk_set_c128_arithmetic(int32_t mode) {
    if (mode != PLK_ARITH_DOUBLE_FLOAT && mode != PLK_ARITH_FP64)
        PLK_FAIL(PLK_ERR_INVALID_ARG, "complex128 arithmetic mode must be 0 (double-float) or 1 (FP64)");
    plk::g_c128_df.store(mode == PLK_ARITH_DOUBLE_FLOAT ? 1 : 0);
    return PLK_OK;
}

PLK_API int plk_get_c128_arithmetic(int32_t *mode) {
    if (!mode) PLK_FAIL(PLK_ERR_INVALID_ARG, "null mode");
    *mode = plk::c128_use_df() ? PLK_ARITH_DOUBLE_FLOAT : PLK_ARITH_FP64;
    return PLK_OK;
}

PLK_API int plk_device_count(int *count) {
    if (!count) PLK_FAIL(PLK_ERR_INVALID_ARG, "null count");
    int c = 0;
    cudaError_t e = cudaGetDeviceCount(&c);
    if (e != cudaSuccess) {
        cudaGetLastError();
        c = 0;
    }
    *count = c;
    return PLK_OK;
}

PLK_API int plk_get_device_info(int device, plk_device_info *out) {
    if (!out) PLK_FAIL(PLK_ERR_INVALID_ARG, "null output");
    DeviceCtx *d = nullptr;
    PLK_TRY(device_ctx(device, &d));
    cudaDeviceProp p;
    PLK_CUDA(cudaGetDeviceProperties(&p, device));
    std::memset(out, 0, sizeof(*out));
    out->device = device;
    out->sm_count = p.multiProcessorCount;
    out->cc_major = p.major;
    out->cc_minor = p.minor;
    out->total_mem = p.totalGlobalMem;
    size_t fr = 0, tot = 0;
    PLK_CUDA(cudaSetDevice(device));
    PLK_CUDA(cudaMemGetInfo(&fr, &tot));
    out->free_mem = fr;
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrClockRate, device);
    out->clock_khz = v;
    cudaDeviceGetAttribute(&v, cudaDevAttrMemoryClockRate, device);
    out->mem_clock_khz = v;
    cudaDeviceGetAttribute(&v, cudaDevAttrGlobalMemoryBusWidth, device);
    out->mem_bus_width = v;
    std::strncpy(out->name, p.name, sizeof(out->name) - 1);
    return PLK_OK;
}

static int alloc_workspace(plk_state s) {
    // partials, results and the ticket counter in one pool block
    const size_t bp = sizeof(double) * kMaxRedValues * kMaxRedBlocks, br = sizeof(double) * kMaxRedValues;
    void *blk = nullptr;
    PLK_TRY(pool_alloc(s->device, &blk, bp + br + 256, s->stream));
    s->ws.d_partials = (double *)blk;
    s->ws.d_result = (double *)((char *)blk + bp);
    s->ws.d_counter = (unsigned int *)((char *)blk + bp + br);
    PLK_CUDA(cudaMemsetAsync(s->ws.d_counter, 0, sizeof(unsigned int) * 4, s->stream));
    PLK_TRY(pinned_get(&s->ws.h_result));
    return PLK_OK;
}

static void free_state(plk_state s) {
    if (!s) return;
    cudaSetDevice(s->device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    if (s->owned && s->data) pool_free(s->data, s->stream);
    if (s->ws.d_partials) pool_free(s->ws.d_partials, s->stream);
    pinned_put(s->ws.h_result);
    s->data = nullptr;
    delete s;
}

PLK_API int plk_state_create(int nq, int dtype, int device, plk_state *out) {
    if (!out) PLK_FAIL(PLK_ERR_INVALID_ARG, "null output handle");
    *out = nullptr;
    if (dtype != PLK_C64 && dtype != PLK_C128) PLK_FAIL(PLK_ERR_INVALID_ARG, "dtype must be PLK_C64 or PLK_C128");
    if (nq < 1 || nq > 40) PLK_FAIL(PLK_ERR_INVALID_ARG, "num_qubits must be in [1, 40]");
    DeviceCtx *d = nullptr;
    PLK_TRY(device_ctx(device, &d));
    PLK_CUDA(cudaSetDevice(device));
    plk_state s = new plk_state_s();
    s->device = device;
    s->nq = nq;
    s->dtype = dtype;
    s->length = 1ULL << nq;
    s->stream = d->stream;
    if (pool_alloc(device, &s->data, s->length * amp_bytes(dtype), s->stream) != PLK_OK) {
        const std::string err = last_error();
        s->data = nullptr;
        delete s;
        PLK_FAIL(PLK_ERR_OUT_OF_MEMORY, "allocation of a " + std::to_string(nq) + "-qubit state failed: " + err);
    }
    int st = alloc_workspace(s);
    if (st == PLK_OK) st = fill_basis(s, 0);
    if (st != PLK_OK) {
        free_state(s);
        return st;
    }
    *out = s;
    return PLK_OK;
}

PLK_API int plk_state_wrap(void *ptr, int nq, int dtype, int device, void *stream, plk_state *out) {
    if (!out || !ptr) PLK_FAIL(PLK_ERR_INVALID_ARG, "null pointer");
    *out = nullptr;
    if (dtype != PLK_C64 && dtype != PLK_C128) PLK_FAIL(PLK_ERR_INVALID_ARG, "bad dtype");
    if (nq < 1 || nq > 40) PLK_FAIL(PLK_ERR_INVALID_ARG, "num_qubits must be in [1, 40]");
    if (((uintptr_t)ptr) % amp_bytes(dtype) != 0) PLK_FAIL(PLK_ERR_INVALID_ARG, "misaligned device pointer");
    DeviceCtx *d = nullptr;
    PLK_TRY(device_ctx(device, &d));
    PLK_CUDA(cudaSetDevice(device));
    plk_state s = new plk_state_s();
    s->device = device;
    s->nq = nq;
    s->dtype = dtype;
    s->length = 1ULL << nq;
    s->data = ptr;
    s->owned = false;
    s->stream = stream ? (cudaStream_t)stream : d->stream;
    int st = alloc_workspace(s);
    if (st != PLK_OK) {
        free_state(s);
        return st;
    }
    *out = s;
    return PLK_OK;
}

PLK_API int plk_state_destroy(plk_state s) {
    if (!s) return PLK_OK;
    free_state(s);
    return PLK_OK;
}

PLK_API int plk_state_get(plk_state s, int *nq, int *dtype, void **ptr) {
    PLK_TRY(check_state(s));
    if (nq) *nq = s->nq;
    if (dtype) *dtype = s->dtype;
    if (ptr) *ptr = s->data;
    return PLK_OK;
}

PLK_API int plk_state_set_stream(plk_state s, void *stream) {
    PLK_TRY(check_state(s));
    DeviceCtx *d = nullptr;
    PLK_TRY(device_ctx(s->device, &d));
    cudaStream_t ns = stream ? (cudaStream_t)stream : d->stream;
    if (ns != s->stream) {
        // keep order: the new stream waits for what is queued on the old one
        cudaEvent_t ev;
        PLK_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        PLK_CUDA(cudaEventRecord(ev, s->stream));
        PLK_CUDA(cudaStreamWaitEvent(ns, ev, 0));
        PLK_CUDA(cudaEventDestroy(ev));
        s->stream = ns;
    }
    return PLK_OK;
}

PLK_API int plk_state_get_stream(plk_state s, void **stream) {
    PLK_TRY(check_state(s));
    if (stream) *stream = (void *)s->stream;
    return PLK_OK;
}

PLK_API int plk_state_synchronize(plk_state s) {
    PLK_TRY(check_state(s));
    PLK_CUDA(cudaStreamSynchronize(s->stream));
    return PLK_OK;
}

PLK_API int plk_state_reset(plk_state s) {
    PLK_TRY(check_state(s));
    PLK_CUDA(cudaSetDevice(s->device));
    return fill_basis(s, 0);
}

PLK_API int plk_state_zero(plk_state s) {
    PLK_TRY(check_state(s));
    PLK_CUDA(cudaSetDevice(s->device));
    PLK_CUDA(cudaMemsetAsync(s->data, 0, s->length * amp_bytes(s->dtype), s->stream));
    return PLK_OK;
}

PLK_API int plk_state_set_basis(plk_state s, uint64_t index) {
    PLK_TRY(check_state(s));
    if (index >= s->length) PLK_FAIL(PLK_ERR_INVALID_ARG, "basis index out of range");
    PLK_CUDA(cudaSetDevice(s->device));
    return fill_basis(s, index);
}

PLK_API int plk_state_set_values(plk_state s, const uint64_t *indices, const void *values, uint64_t count) {
    PLK_TRY(check_state(s));
    if (count > 0 && (!indices || !values)) PLK_FAIL(PLK_ERR_INVALID_ARG, "null indices/values");
    for (uint64_t i = 0; i < count; i++)
        if (indices[i] >= s->length) PLK_FAIL(PLK_ERR_INVALID_ARG, "index out of range in setStateVector");
    PLK_CUDA(cudaSetDevice(s->device));
    PLK_CUDA(cudaMemsetAsync(s->data, 0, s->length * amp_bytes(s->dtype), s->stream));
    if (count == 0) return PLK_OK;
    void *d_idx = nullptr, *d_val = nullptr;
    PLK_CUDA(cudaMallocAsync(&d_idx, count * sizeof(uint64_t), s->stream));
    PLK_CUDA(cudaMallocAsync(&d_val, count * amp_bytes(s->dtype), s->stream));
    PLK_CUDA(cudaMemcpyAsync(d_idx, indices, count * sizeof(uint64_t), cudaMemcpyHostToDevice, s->stream));
    PLK_CUDA(cudaMemcpyAsync(d_val, values, count * amp_bytes(s->dtype), cudaMemcpyHostToDevice, s->stream));
    const int g = elem_grid(s, count);
    if (s->dtype == PLK_C64)
        k_scatter<float2><<<g, kThreads, 0, s->stream>>>((float2 *)s->data, (const uint64_t *)d_idx,
                                                           (const float2 *)d_val, count);
    else
        k_scatter<double2><<<g, kThreads, 0, s->stream>>>((double2 *)s->data, (const uint64_t *)d_idx,
                                                            (const double2 *)d_val, count);
    PLK_CHECK_LAUNCH();
    PLK_CUDA(cudaFreeAsync(d_idx, s->stream));
    PLK_CUDA(cudaFreeAsync(d_val, s->stream));
    PLK_CUDA(cudaStreamSynchronize(s->stream)); // host buffers may go away after return
    return PLK_OK;
}

PLK_API int plk_state_h2d(plk_state s, const void *host, uint64_t length) {
    PLK_TRY(check_state(s));
    if (length != s->length) PLK_FAIL(PLK_ERR_INVALID_ARG, "length does not match the state size");
    if (!host) PLK_FAIL(PLK_ERR_INVALID_ARG, "null host buffer");
    PLK_CUDA(cudaSetDevice(s->device));
    PLK_CUDA(cudaMemcpyAsync(s->data, host, length * amp_bytes(s->dtype), cudaMemcpyHostToDevice, s->stream));
    PLK_CUDA(cudaStreamSynchronize(s->stream));
    return PLK_OK;
}

PLK_API int plk_state_d2h(plk_state s, void *host, uint64_t length) {
    PLK_TRY(check_state(s));
    if (length != s->length) PLK_FAIL(PLK_ERR_INVALID_ARG, "length does not match the state size");
    if (!host) PLK_FAIL(PLK_ERR_INVALID_ARG, "null host buffer");
    PLK_CUDA(cudaSetDevice(s->device));
    PLK_CUDA(cudaMemcpyAsync(host, s->data, length * amp_bytes(s->dtype), cudaMemcpyDeviceToHost, s->stream));
    PLK_CUDA(cudaStreamSynchronize(s->stream));
    return PLK_OK;
}

PLK_API int plk_state_h2d_async(plk_state s, const void *host, uint64_t length) {
    PLK_TRY(check_state(s));
    if (length != s->length) PLK_FAIL(PLK_ERR_INVALID_ARG, "length does not match the state size");
    if (!host) PLK_FAIL(PLK_ERR_INVALID_ARG, "null host buffer");
    PLK_CUDA(cudaSetDevice(s->device));
    PLK_CUDA(cudaMemcpyAsync(s->data, host, length * amp_bytes(s->dtype), cudaMemcpyHostToDevice, s->stream));
    return PLK_OK;
}

PLK_API int plk_state_d2h_async(plk_state s, void *host, uint64_t length) {
    PLK_TRY(check_state(s));
    if (length != s->length) PLK_FAIL(PLK_ERR_INVALID_ARG, "length does not match the state size");
    if (!host) PLK_FAIL(PLK_ERR_INVALID_ARG, "null host buffer");
    PLK_CUDA(cudaSetDevice(s->device));
    PLK_CUDA(cudaMemcpyAsync(host, s->data, length * amp_bytes(s->dtype), cudaMemcpyDeviceToHost, s->stream));
    return PLK_OK;
}

PLK_API int plk_state_copy(plk_state dst, plk_state src) {
    PLK_TRY(check_state(dst));
    PLK_TRY(check_state(src));
    if (dst->nq != src->nq || dst->dtype != src->dtype)
        PLK_FAIL(PLK_ERR_INVALID_ARG, "states differ in size or precision");
    if (dst == src) return PLK_OK;
    PLK_CUDA(cudaSetDevice(dst->device));
    PLK_TRY(order_after(dst, src));
    PLK_CUDA(cudaMemcpyAsync(dst->data, src->data, dst->length * amp_bytes(dst->dtype), cudaMemcpyDeviceToDevice,
                             dst->stream));
    PLK_TRY(order_after(src, dst));
    return PLK_OK;
}

PLK_API int plk_state_axpy(plk_state y, double are, double aim, plk_state x) {
    PLK_TRY(check_state(y));
    PLK_TRY(check_state(x));
    if (y->nq != x->nq || y->dtype != x->dtype) PLK_FAIL(PLK_ERR_INVALID_ARG, "states differ in size or precision");
    PLK_CUDA(cudaSetDevice(y->device));
    PLK_TRY(order_after(y, x));
    const int g = elem_grid(y, (y->length + 1) / 2);
    const bool real = aim == 0.0;
    if (y->dtype == PLK_C64) {
        if (real)
            k_axpy<float2, float, true><<<g, kThreads, 0, y->stream>>>((float2 *)y->data, (const float2 *)x->data,
                                                                        (float)are, 0.0f, y->length);
        else
            k_axpy<float2, float, false><<<g, kThreads, 0, y->stream>>>((float2 *)y->data, (const float2 *)x->data,
                                                                         (float)are, (float)aim, y->length);
    } else {
        if (real)
            k_axpy<double2, double, true><<<g, kThreads, 0, y->stream>>>((double2 *)y->data, (const double2 *)x->data,
                                                                          are, 0.0, y->length);
        else
            k_axpy<double2, double, false><<<g, kThreads, 0, y->stream>>>((double2 *)y->data,
                                                                           (const double2 *)x->data, are, aim,
                                                                           y->length);
    }
    PLK_CHECK_LAUNCH();
    PLK_TRY(order_after(x, y));
    return PLK_OK;
}

} // extern "C"
