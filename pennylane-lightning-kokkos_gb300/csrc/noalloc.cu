// noalloc.cu — PauliZ / Identity expectation values without device allocation.
//
// Who needs this: callers that must not allocate device memory.  A caller
// whose device memory belongs to another allocator — a framework's caching
// allocator, or a serving process running under a fixed memory budget — cannot
// call cudaMalloc/cudaFree: those bypass the budget and synchronize the whole
// device.  The regular entry points keep reduction workspace in each
// plk_state (allocated at creation); this one works on a bare, caller-owned
// device state and writes into a caller-owned device buffer, with no plk_state
// and no allocation at all.
//
// Scratch: g_noalloc_scratch below, a file-scope __device__ array of
// kNoAllocScratchBytes = 256 + 16 x 256 x 8 bytes (32.25 KiB): a 256-byte slot
// for the blocks' ticket counter, then kNoAllocMaxValues x kNoAllocMaxBlocks
// FP64 partial sums.  Every GPU that loads this library holds the array until
// the process exits.  All calls share it and it keeps the last call's
// contents, so each call clears the counter first and rewrites every partial
// it reads.  Calls that overlap on the GPU (different streams, or host threads
// without ordering between them) race on the array and return wrong values.
//
// Set-up: host code cannot use the array's name as a device address, so the
// first call on a device (with that device current) looks the address up with
// cudaGetSymbolAddress and caches it for that device; make that first call
// before any stream capture on the device.
#include <algorithm>
#include <mutex>
#include <string>

#include "reduce.cuh"

namespace plk {

constexpr int kNoAllocMaxValues = 16;
constexpr int kNoAllocMaxBlocks = 256;
constexpr size_t kNoAllocCounterBytes = 256;
constexpr size_t kNoAllocScratchBytes =
    kNoAllocCounterBytes + sizeof(double) * (size_t)kNoAllocMaxValues * kNoAllocMaxBlocks;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {
std::mutex g_noalloc_mutex;
void *g_noalloc_ptr[64] = {nullptr};
} // namespace

struct ZMasks {
    uint64_t z[kNoAllocMaxValues];
};

// One pass over the state: value v = sum_k |psi_k|^2 (-1)^popcount(k & z_v).
template <class T>
__global__ void __launch_bounds__(kThreads)
    k_expval_diag_noalloc(const c2_t<T> *__restrict__ sv, uint64_t n, const ZMasks zm, int nv,
                          unsigned char *__restrict__ scratch, double *__restrict__ out) {
    double acc[kNoAllocMaxValues];
#pragma unroll
    for (int v = 0; v < kNoAllocMaxValues; v++) acc[v] = 0.0;
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += step) {
        const c2_t<T> a = sv[k];
        const double p = (double)a.x * a.x + (double)a.y * a.y;
#pragma unroll
        for (int v = 0; v < kNoAllocMaxValues; v++) acc[v] += (__popcll(k & zm.z[v]) & 1) ? -p : p;
    }
    auto *counter = reinterpret_cast<unsigned int *>(scratch);
    auto *partials = reinterpret_cast<double *>(scratch + kNoAllocCounterBytes);
    block_reduce_finish<kNoAllocMaxValues>(acc, partials, out, counter, 1.0, nv);
}

static int noalloc_scratch(int device, void **out) {
    std::lock_guard<std::mutex> lk(g_noalloc_mutex);
    if (!g_noalloc_ptr[device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            PLK_FAIL(PLK_ERR_CUDA, std::string("cudaGetSymbolAddress of the no-allocation scratch failed: ") +
                                       cudaGetErrorString(e));
        }
        g_noalloc_ptr[device] = p;
    }
    *out = g_noalloc_ptr[device];
    return PLK_OK;
}

} // namespace plk

using namespace plk;

extern "C" {

PLK_API int plk_expval_pauliz_noalloc(const void *state, int32_t num_qubits, int32_t dtype, int32_t count,
                                      const int64_t *wires, double *out, void *cuda_stream) {
    if (!state || !wires || !out) PLK_FAIL(PLK_ERR_INVALID_ARG, "null state, wires or output pointer");
    if (num_qubits < 1 || num_qubits > 40) PLK_FAIL(PLK_ERR_INVALID_ARG, "num_qubits must be in [1, 40]");
    if (dtype != PLK_C64 && dtype != PLK_C128) PLK_FAIL(PLK_ERR_INVALID_ARG, "dtype must be PLK_C64 or PLK_C128");
    if (count < 1 || count > kNoAllocMaxValues)
        PLK_FAIL(PLK_ERR_INVALID_ARG, "count " + std::to_string(count) + " is outside [1, " +
                                          std::to_string(kNoAllocMaxValues) +
                                          "]: the no-allocation scratch holds at most " +
                                          std::to_string(kNoAllocMaxValues) + " values per call");
    if (((uintptr_t)state) % amp_bytes(dtype) != 0 || ((uintptr_t)out) % sizeof(double) != 0)
        PLK_FAIL(PLK_ERR_INVALID_ARG, "misaligned state or output pointer");
    ZMasks zm{};
    for (int i = 0; i < count; i++) {
        if (wires[i] < -1 || wires[i] >= num_qubits)
            PLK_FAIL(PLK_ERR_INVALID_ARG, "wire " + std::to_string(wires[i]) + " out of range (-1 = Identity)");
        zm.z[i] = wires[i] < 0 ? 0ULL : (1ULL << (num_qubits - 1 - wires[i]));
    }
    int device = 0;
    PLK_CUDA(cudaGetDevice(&device));
    if (device < 0 || device >= 64) PLK_FAIL(PLK_ERR_INVALID_ARG, "device id out of range");
    void *scratch = nullptr;
    PLK_TRY(noalloc_scratch(device, &scratch));
    int sms = 0;
    PLK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    const uint64_t n = 1ULL << num_qubits;
    uint64_t grid = (n + kThreads - 1) / kThreads;
    const uint64_t cap = std::min<uint64_t>((uint64_t)kNoAllocMaxBlocks, (uint64_t)sms * 2);
    if (grid > cap) grid = cap;
    if (grid < 1) grid = 1;
    cudaStream_t st = (cudaStream_t)cuda_stream;
    PLK_CUDA(cudaMemsetAsync(scratch, 0, kNoAllocCounterBytes, st)); // ticket counter starts at zero
    auto *scr = static_cast<unsigned char *>(scratch);
    if (dtype == PLK_C64)
        k_expval_diag_noalloc<float><<<(unsigned)grid, kThreads, 0, st>>>((const float2 *)state, n, zm, count, scr, out);
    else
        k_expval_diag_noalloc<double><<<(unsigned)grid, kThreads, 0, st>>>((const double2 *)state, n, zm, count, scr,
                                                                            out);
    PLK_CHECK_LAUNCH();
    return PLK_OK;
}

} // extern "C"
