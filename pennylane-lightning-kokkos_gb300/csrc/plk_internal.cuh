// plk_internal.cuh — shared internals of the GB300 state-vector core.
//
// Layout in HBM: one contiguous array of 2^n amplitudes per state, float2
// (complex64) or double2 (complex128), 256-byte aligned by cudaMalloc.  Wire 0
// is the most significant index bit; a gate on wire w touches bit
// b = n - 1 - w.  Every kernel addresses amplitudes through a group index g:
// the base index of group g is g with zero bits inserted at the sorted target
// bit positions, and local index i (bit K-1-j <-> wires[j]) adds off[i].
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>

#include "plk_gb300.h"

namespace plk {

// ----------------------------------------------------------------------------
// errors
// ----------------------------------------------------------------------------
void set_error(const std::string &msg);
const std::string &last_error();

struct Error {
    int status;
    std::string msg;
};

#define PLK_FAIL(st, msg)                                                      \
    do {                                                                       \
        ::plk::set_error(msg);                                                 \
        return (st);                                                           \
    } while (0)

#define PLK_CUDA(call)                                                         \
    do {                                                                       \
        cudaError_t e_ = (call);                                               \
        if (e_ != cudaSuccess) {                                               \
            ::plk::set_error(std::string("CUDA error: ") + cudaGetErrorString(e_) + \
                             " at " + __FILE__ + ":" + std::to_string(__LINE__)); \
            return (e_ == cudaErrorMemoryAllocation) ? PLK_ERR_OUT_OF_MEMORY   \
                                                     : PLK_ERR_CUDA;           \
        }                                                                      \
    } while (0)

#define PLK_TRY(call)                                                          \
    do {                                                                       \
        int st_ = (call);                                                      \
        if (st_ != PLK_OK) return st_;                                         \
    } while (0)

#define PLK_CHECK_LAUNCH() PLK_CUDA(cudaGetLastError())

// ----------------------------------------------------------------------------
// devices and launch geometry
// ----------------------------------------------------------------------------
struct DeviceCtx {
    int sm_count = 0;
    int max_threads_per_sm = 0;
    cudaStream_t stream = nullptr; // library stream of this device
    cudaMemPool_t pool = nullptr;  // stream-ordered pool for state buffers (keeps freed blocks mapped)
};
int device_ctx(int device, DeviceCtx **out);

// State buffers come from the device's pool: allocation on `stream`, ready
// for any stream on return; release is stream ordered.
int pool_alloc(int device, void **ptr, size_t bytes, cudaStream_t stream);
void pool_free(void *ptr, cudaStream_t stream);

// Pool block released (stream-ordered) when the guard goes out of scope, on
// every return path.
struct PoolBuf {
    void *p = nullptr;
    cudaStream_t st = nullptr;
    explicit PoolBuf(cudaStream_t s) : st(s) {}
    PoolBuf(const PoolBuf &) = delete;
    PoolBuf &operator=(const PoolBuf &) = delete;
    ~PoolBuf() { pool_free(p, st); }
    template <class U> U *as() const { return static_cast<U *>(p); }
};


constexpr int kThreads = 256;
// Reductions use a fixed grid (a function of the device only) so that the
// order of the FP64 partial sums, hence the result bits, never changes.
constexpr int kMaxRedBlocks = 1024;
constexpr int kMaxRedValues = 64; // values reduced together in one pass

// ----------------------------------------------------------------------------
// states
// ----------------------------------------------------------------------------
struct Workspace {
    double *d_partials = nullptr;   // [kMaxRedValues][kMaxRedBlocks]
    double *d_result = nullptr;     // [kMaxRedValues]
    unsigned int *d_counter = nullptr;
    double *h_result = nullptr;     // pinned [kMaxRedValues]
};

} // namespace plk

struct plk_state_s {
    int device = 0;
    int nq = 0;
    int dtype = PLK_C128;
    uint64_t length = 0;
    void *data = nullptr;
    bool owned = true;
    cudaStream_t stream = nullptr;
    plk::Workspace ws;
};

namespace plk {

inline size_t amp_bytes(int dtype) { return dtype == PLK_C64 ? 8 : 16; }

int check_state(plk_state s);
int check_wires(plk_state s, const int64_t *wires, int nw);
// Make `s`'s stream wait for work queued so far on `other`'s stream.
int order_after(plk_state s, plk_state other);
int red_grid(const plk_state_s *s, uint64_t work_items);
int device_sm_count(int device);
// Grid of a reduction kernel: the blocks that fit on the device at once for
// this kernel (a whole number per SM, so there is no partial last wave),
// at most kMaxRedBlocks and no more than the work needs.  A function of the
// kernel, the device and the size only, so the partial-sum order is fixed.
template <class Kern>
int red_grid_k(const plk_state_s *s, Kern kernel, uint64_t work_items, size_t dyn_smem = 0) {
    const int sms = device_sm_count(s->device);
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, kThreads, dyn_smem) != cudaSuccess || occ < 1) {
        cudaGetLastError();
        occ = 1;
    }
    int per_sm = kMaxRedBlocks / (sms > 0 ? sms : 1);
    if (per_sm > occ) per_sm = occ;
    if (per_sm < 1) per_sm = 1;
    uint64_t want = (work_items + kThreads - 1) / kThreads;
    const uint64_t cap = (uint64_t)(sms > 0 ? sms : 1) * per_sm;
    if (want > cap) want = cap;
    return want < 1 ? 1 : (int)want;
}
// Grid for element-wise / grid-stride kernels on this state's device.
int elem_grid(plk_state s, uint64_t work_items);
// Set the state to basis vector |index> (InitView / setBasisStateFunctor).
int fill_basis(plk_state s, uint64_t index);
// complex128 arithmetic on the FP32 pipe (default) or native FP64
// (environment PLK_C128_ARITH=fp64).
bool c128_use_df();

// complex64 dense matrices on 5 or 6 wires on the tensor cores (dense_tc.cu)
// unless plk_set_dense_tensor_cores(0)
bool dense_tc_enabled();
struct Masks;
int launch_dense_tc(plk_state s, const float2 *U, const uint64_t *hoff, const Masks &gm, int K);

// ----------------------------------------------------------------------------
// complex arithmetic on float2 / double2
// ----------------------------------------------------------------------------
template <class T> struct C2;
template <> struct C2<float> { using type = float2; };
template <> struct C2<double> { using type = double2; };
template <class T> using c2_t = typename C2<T>::type;

template <class V> __host__ __device__ __forceinline__ V mk(decltype(V::x) re, decltype(V::x) im) {
    V r;
    r.x = re;
    r.y = im;
    return r;
}
template <class V> __host__ __device__ __forceinline__ V cmul(V a, V b) {
    return mk<V>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <class V> __host__ __device__ __forceinline__ V cadd(V a, V b) { return mk<V>(a.x + b.x, a.y + b.y); }
template <class V> __host__ __device__ __forceinline__ V csub(V a, V b) { return mk<V>(a.x - b.x, a.y - b.y); }
template <class V, class T> __host__ __device__ __forceinline__ V rmul(T s, V a) { return mk<V>(s * a.x, s * a.y); }
template <class V> __host__ __device__ __forceinline__ V cneg(V a) { return mk<V>(-a.x, -a.y); }
template <class V> __host__ __device__ __forceinline__ V mul_i(V a) { return mk<V>(-a.y, a.x); }   // i*a
template <class V> __host__ __device__ __forceinline__ V mul_mi(V a) { return mk<V>(a.y, -a.x); }  // -i*a

// ----------------------------------------------------------------------------
// group index maps
// ----------------------------------------------------------------------------
// Insert zero bits at m sorted bit positions: base = OR_j ((g << j) & mask_j),
// with mask_0 = ones below p0, mask_j = ones in (p_{j-1}, p_j), mask_m = ones
// above p_{m-1} (the parity_low/middle/high masks of the reference functors).
constexpr int kMaxDenseWires = 12;
struct Masks {
    uint64_t m[kMaxDenseWires + 1];
};
Masks make_masks(const int *sorted_bits, int count);

template <int K> __device__ __forceinline__ uint64_t group_base(uint64_t g, const Masks &mk) {
    uint64_t r = g & mk.m[0];
#pragma unroll
    for (int j = 1; j <= K; j++) r |= (g << j) & mk.m[j];
    return r;
}

} // namespace plk
