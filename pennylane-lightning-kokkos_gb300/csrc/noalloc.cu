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
// kNoAllocScratchBytes = 256 + 16 x 1024 x 8 bytes (128.25 KiB): a 256-byte
// slot for the blocks' ticket counter, then kNoAllocMaxValues x
// kNoAllocMaxBlocks FP64 partial sums.  Every GPU that loads this library holds the array until
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

#include "expval_diag.cuh"

namespace plk {

constexpr int kNoAllocMaxValues = 16;
constexpr int kNoAllocMaxBlocks = 1024;
constexpr size_t kNoAllocCounterBytes = 256;
constexpr size_t kNoAllocScratchBytes =
    kNoAllocCounterBytes + sizeof(double) * (size_t)kNoAllocMaxValues * kNoAllocMaxBlocks;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {
std::mutex g_noalloc_mutex;
void *g_noalloc_ptr[64] = {nullptr};
} // namespace

// The same one-pass kernel as the regular entry points for single-wire
// PauliZ / Identity values (k_expval_zbits, expval_diag.cuh), with its
// partial sums (value v of block b at v * grid + b) and ticket counter in the
// fixed scratch array and the results written to the caller's buffer.  The
// grid is the kernel's resident blocks per SM times the SM count (at most
// kNoAllocMaxBlocks), found with the occupancy API, which allocates nothing.
template <class T>
static int launch_noalloc(const void *state, uint64_t n, const ZBits &zb, int nv, unsigned char *scr, double *out,
                          cudaStream_t st, int sms) {
    constexpr int M = sizeof(T) == 4 ? 5 : 4; // steps per lane per chunk: 2^M
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_expval_zbits<T, M>, kThreads, 0) != cudaSuccess ||
        occ < 1) {
        cudaGetLastError();
        occ = 1;
    }
    const uint64_t chunks = (n + ((uint64_t)32 << M) - 1) / ((uint64_t)32 << M);
    uint64_t grid = (chunks * 32 + kThreads - 1) / kThreads; // one warp per chunk
    const uint64_t cap = std::min<uint64_t>((uint64_t)kNoAllocMaxBlocks, (uint64_t)sms * (uint64_t)occ);
    if (grid > cap) grid = cap;
    if (grid < 1) grid = 1;
    auto *counter = reinterpret_cast<unsigned int *>(scr);
    auto *partials = reinterpret_cast<double *>(scr + kNoAllocCounterBytes);
    k_expval_zbits<T, M><<<(unsigned)grid, kThreads, 0, st>>>((const c2_t<T> *)state, n, zb, nv, partials, out,
                                                              counter);
    PLK_CHECK_LAUNCH();
    return PLK_OK;
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
    ZBits zb{};
    for (int i = 0; i < count; i++) {
        if (wires[i] < -1 || wires[i] >= num_qubits)
            PLK_FAIL(PLK_ERR_INVALID_ARG, "wire " + std::to_string(wires[i]) + " out of range (-1 = Identity)");
        zb.b[i] = wires[i] < 0 ? (int8_t)-1 : (int8_t)(num_qubits - 1 - wires[i]);
    }
    int device = 0;
    PLK_CUDA(cudaGetDevice(&device));
    if (device < 0 || device >= 64) PLK_FAIL(PLK_ERR_INVALID_ARG, "device id out of range");
    void *scratch = nullptr;
    PLK_TRY(noalloc_scratch(device, &scratch));
    int sms = 0;
    PLK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    const uint64_t n = 1ULL << num_qubits;
    cudaStream_t st = (cudaStream_t)cuda_stream;
    PLK_CUDA(cudaMemsetAsync(scratch, 0, kNoAllocCounterBytes, st)); // ticket counter starts at zero
    auto *scr = static_cast<unsigned char *>(scratch);
    return dtype == PLK_C64 ? launch_noalloc<float>(state, n, zb, count, scr, out, st, sms)
                            : launch_noalloc<double>(state, n, zb, count, scr, out, st, sms);
}

} // extern "C"
