// measure.cu — probabilities, CDF and sampling.
//
// Replaces MeasuresKokkos::probs / probs(wires) / generate_samples
// (simulator/MeasuresKokkos.hpp:389-569) and getProbFunctor, getCDFFunctor,
// Sampler, getSubProbFunctor and the transpose functors
// (simulator/MeasuresFunctors.hpp).
//
//  - probs(): |psi_k|^2 in FP64.
//  - probs(wires): marginals computed directly in the requested wire order
//    (no separate transpose pass); small outputs use per-block shared-memory
//    histograms summed in block order, large outputs one thread per bin.
//  - CDF: exclusive scan in FP64 over fixed 1024-amplitude tiles (tile sums,
//    a serial scan of the tile sums, then per-tile scans).
//  - Sampler: the reference's search (index 0 if U <= cdf[1], else a binary
//    search over [1, N] with cdf[N] = 1), so identical CDF and uniforms give
//    identical indices; uniforms come from Philox-4x32-10 (Salmon, Moraes,
//    Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11).
#include <algorithm>
#include <cstring>
#include <vector>

#include "df.cuh"
#include "plk_internal.cuh"

namespace plk {

template <class T>
__global__ void __launch_bounds__(kThreads) k_probs(const c2_t<T> *__restrict__ sv, double *__restrict__ p, uint64_t n) {
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += step) {
        const DF q = df_norm2(to_cdf(sv[k])); // |psi_k|^2 on the FP32 pipe, one FP64 add
        p[k] = df_result(q.hi, q.lo);
    }
}

// bin index of amplitude k in the requested wire order: output bit (m-1-j)
// is amplitude bit rev[j].
__device__ __forceinline__ uint32_t bin_of(uint64_t k, const int *rev, int m) {
    uint32_t o = 0;
    for (int j = 0; j < m; j++) o |= (uint32_t)((k >> rev[j]) & 1ULL) << (m - 1 - j);
    return o;
}

struct WireList {
    int rev[32];
    int m;
};

// per-block histogram (m <= 12), partial[block][bin]
template <class T>
__global__ void __launch_bounds__(kThreads)
    k_marginal_hist(const c2_t<T> *__restrict__ sv, uint64_t n, WireList w, double *__restrict__ partial) {
    extern __shared__ double hist[];
    const int nb = 1 << w.m;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) hist[i] = 0.0;
    __syncthreads();
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += step) {
        const c2_t<T> a = sv[k];
        atomicAdd(&hist[bin_of(k, w.rev, w.m)], (double)a.x * a.x + (double)a.y * a.y);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nb; i += blockDim.x) partial[(size_t)blockIdx.x * nb + i] = hist[i];
}

__global__ void k_sum_partials(const double *__restrict__ partial, int nblocks, int nb, double *__restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb) return;
    double s = 0.0;
    for (int b = 0; b < nblocks; b++) s += partial[(size_t)b * nb + i];
    out[i] = s;
}

// one thread per output bin: sums the 2^(n-m) amplitudes of the bin in order;
// rest index r is deposited into the bit positions that are not measured.
struct RestBits {
    int bit[64];
    int count;
};

template <class T>
__global__ void __launch_bounds__(kThreads)
    k_marginal_gather(const c2_t<T> *__restrict__ sv, RestBits rb, const uint64_t *__restrict__ bin_off, uint64_t nrest,
                      uint64_t nbins, double *__restrict__ out) {
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t o = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; o < nbins; o += step) {
        const uint64_t off = bin_off[o];
        double s = 0.0;
        for (uint64_t r = 0; r < nrest; r++) {
            uint64_t base = 0;
            for (int j = 0; j < rb.count; j++) base |= ((r >> j) & 1ULL) << rb.bit[j];
            const c2_t<T> a = sv[base | off];
            s += (double)a.x * a.x + (double)a.y * a.y;
        }
        out[o] = s;
    }
}

// ------------------------------------------------------------------ CDF --
constexpr int kScanTile = 1024;

template <class T>
__global__ void __launch_bounds__(kThreads)
    k_tile_sums(const c2_t<T> *__restrict__ sv, uint64_t n, double *__restrict__ tile_sum) {
    // one block per tile, fixed-order tree inside the block
    __shared__ double sh[kThreads];
    const uint64_t t = blockIdx.x;
    double s = 0.0;
    for (int j = threadIdx.x; j < kScanTile; j += kThreads) {
        const uint64_t k = t * kScanTile + j;
        if (k < n) {
            const c2_t<T> a = sv[k];
            s += (double)a.x * a.x + (double)a.y * a.y;
        }
    }
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = kThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) tile_sum[t] = sh[0];
}

// exclusive scan of the tile sums (serial, in order; ntiles = N / 1024)
__global__ void k_scan_tiles(double *__restrict__ tile_sum, uint64_t ntiles) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double run = 0.0;
    for (uint64_t t = 0; t < ntiles; t++) {
        const double v = tile_sum[t];
        tile_sum[t] = run;
        run += v;
    }
}

// per tile: cdf[k] = tile_offset + exclusive prefix inside the tile
template <class T>
__global__ void __launch_bounds__(kThreads)
    k_tile_scan(const c2_t<T> *__restrict__ sv, uint64_t n, const double *__restrict__ tile_off, double *__restrict__ cdf) {
    constexpr int PER = kScanTile / kThreads; // 4 amplitudes per thread
    __shared__ double sh[kThreads];
    const uint64_t t = blockIdx.x;
    double v[PER];
    double local = 0.0;
#pragma unroll
    for (int j = 0; j < PER; j++) {
        const uint64_t k = t * kScanTile + (uint64_t)threadIdx.x * PER + j;
        double p = 0.0;
        if (k < n) {
            const c2_t<T> a = sv[k];
            p = (double)a.x * a.x + (double)a.y * a.y;
        }
        v[j] = p;
        local += p;
    }
    // inclusive Hillis-Steele scan of per-thread sums (fixed order)
    sh[threadIdx.x] = local;
    __syncthreads();
    for (int w = 1; w < kThreads; w <<= 1) {
        const double add = threadIdx.x >= (unsigned)w ? sh[threadIdx.x - w] : 0.0;
        __syncthreads();
        sh[threadIdx.x] += add;
        __syncthreads();
    }
    double run = tile_off[t] + (sh[threadIdx.x] - local);
#pragma unroll
    for (int j = 0; j < PER; j++) {
        const uint64_t k = t * kScanTile + (uint64_t)threadIdx.x * PER + j;
        if (k < n) cdf[k] = run;
        run += v[j];
    }
}

// ------------------------------------------------------------- sampling --
__device__ __forceinline__ uint64_t search_cdf(const double *__restrict__ cdf, uint64_t n, double U) {
    if (n < 2 || U <= cdf[1]) return 0;
    uint64_t lo = 1, hi = n;
    while (hi - lo > 1) {
        const uint64_t mid = hi - ((hi - lo) >> 1);
        const double ct = (mid == n) ? 1.0 : cdf[mid];
        if (ct < U) lo = mid;
        else hi = mid;
    }
    return hi - 1;
}

__global__ void k_sample(const double *__restrict__ cdf, uint64_t n, int nq, const double *__restrict__ u,
                         uint64_t shots, int64_t *__restrict__ bits) {
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < shots; s += step) {
        const uint64_t idx = search_cdf(cdf, n, u[s]);
        for (int j = 0; j < nq; j++) bits[s * nq + (nq - 1 - j)] = (int64_t)((idx >> j) & 1ULL);
    }
}

// Philox-4x32-10: 10 rounds of the Philox S-box on a 128-bit counter with a
// 64-bit key (constants from the SC'11 paper).
__host__ __device__ inline void philox4x32_10(uint32_t ctr[4], uint32_t key[2]) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; r++) {
        const uint64_t p0 = (uint64_t)M0 * ctr[0];
        const uint64_t p1 = (uint64_t)M1 * ctr[2];
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        const uint32_t n0 = hi1 ^ ctr[1] ^ k0, n1 = lo1, n2 = hi0 ^ ctr[3] ^ k1, n3 = lo0;
        ctr[0] = n0;
        ctr[1] = n1;
        ctr[2] = n2;
        ctr[3] = n3;
        k0 += W0;
        k1 += W1;
    }
}

// uniform double in [0, 1) with 53 random bits from two 32-bit words
__host__ __device__ inline double u53(uint32_t a, uint32_t b) {
    const uint64_t x = ((uint64_t)(a >> 5) << 26) | (uint64_t)(b >> 6);
    return (double)x * (1.0 / 9007199254740992.0);
}

__global__ void k_philox_uniforms(uint64_t seed, uint64_t shots, double *__restrict__ u) {
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; 2 * i < shots; i += step) {
        uint32_t ctr[4] = {(uint32_t)i, (uint32_t)(i >> 32), 0x51ED270Bu, 0u};
        uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
        philox4x32_10(ctr, key);
        u[2 * i] = u53(ctr[0], ctr[1]);
        if (2 * i + 1 < shots) u[2 * i + 1] = u53(ctr[2], ctr[3]);
    }
}

// ------------------------------------------------------------- helpers --
template <class T> static int cdf_device(plk_state s, double *d_cdf) {
    const uint64_t n = s->length;
    const uint64_t ntiles = (n + kScanTile - 1) / kScanTile;
    double *d_tiles = nullptr;
    PLK_CUDA(cudaMallocAsync((void **)&d_tiles, sizeof(double) * ntiles, s->stream));
    auto *sv = (const c2_t<T> *)s->data;
    k_tile_sums<T><<<(unsigned)ntiles, kThreads, 0, s->stream>>>(sv, n, d_tiles);
    PLK_CHECK_LAUNCH();
    k_scan_tiles<<<1, 32, 0, s->stream>>>(d_tiles, ntiles);
    PLK_CHECK_LAUNCH();
    k_tile_scan<T><<<(unsigned)ntiles, kThreads, 0, s->stream>>>(sv, n, d_tiles, d_cdf);
    PLK_CHECK_LAUNCH();
    PLK_CUDA(cudaFreeAsync(d_tiles, s->stream));
    return PLK_OK;
}

static int cdf_any(plk_state s, double *d_cdf) {
    return s->dtype == PLK_C64 ? cdf_device<float>(s, d_cdf) : cdf_device<double>(s, d_cdf);
}

static int sample_with_uniforms_dev(plk_state s, const double *d_u, uint64_t shots, int64_t *out_bits) {
    double *d_cdf = nullptr;
    int64_t *d_bits = nullptr;
    PLK_CUDA(cudaMallocAsync((void **)&d_cdf, sizeof(double) * s->length, s->stream));
    PLK_TRY(cdf_any(s, d_cdf));
    PLK_CUDA(cudaMallocAsync((void **)&d_bits, sizeof(int64_t) * shots * s->nq, s->stream));
    const int grid = elem_grid(s, shots);
    k_sample<<<grid, kThreads, 0, s->stream>>>(d_cdf, s->length, s->nq, d_u, shots, d_bits);
    PLK_CHECK_LAUNCH();
    PLK_CUDA(cudaMemcpyAsync(out_bits, d_bits, sizeof(int64_t) * shots * s->nq, cudaMemcpyDeviceToHost, s->stream));
    PLK_CUDA(cudaFreeAsync(d_cdf, s->stream));
    PLK_CUDA(cudaFreeAsync(d_bits, s->stream));
    PLK_CUDA(cudaStreamSynchronize(s->stream));
    return PLK_OK;
}

template <class T> static int marginal_impl(plk_state s, const int64_t *wires, int m, double *out) {
    WireList wl;
    wl.m = m;
    for (int j = 0; j < m; j++) wl.rev[j] = s->nq - 1 - (int)wires[j];
    const uint64_t nb = 1ULL << m;
    auto *sv = (const c2_t<T> *)s->data;
    double *d_out = nullptr;
    PLK_CUDA(cudaMallocAsync((void **)&d_out, sizeof(double) * nb, s->stream));
    if (m <= 12) {
        DeviceCtx *d = nullptr;
        PLK_TRY(device_ctx(s->device, &d));
        const int grid = std::max(1, std::min<int>((int)((s->length + kThreads - 1) / kThreads), d->sm_count * 2));
        double *d_part = nullptr;
        PLK_CUDA(cudaMallocAsync((void **)&d_part, sizeof(double) * nb * grid, s->stream));
        k_marginal_hist<T><<<grid, kThreads, sizeof(double) * nb, s->stream>>>(sv, s->length, wl, d_part);
        PLK_CHECK_LAUNCH();
        k_sum_partials<<<(unsigned)((nb + 255) / 256), 256, 0, s->stream>>>(d_part, grid, (int)nb, d_out);
        PLK_CHECK_LAUNCH();
        PLK_CUDA(cudaFreeAsync(d_part, s->stream));
    } else {
        RestBits rb;
        rb.count = 0;
        for (int b = 0; b < s->nq; b++) {
            bool measured = false;
            for (int j = 0; j < m; j++) measured |= (wl.rev[j] == b);
            if (!measured) rb.bit[rb.count++] = b;
        }
        std::vector<uint64_t> boff(nb);
        for (uint64_t o = 0; o < nb; o++) {
            uint64_t off = 0;
            for (int j = 0; j < m; j++)
                if ((o >> (m - 1 - j)) & 1) off |= 1ULL << wl.rev[j];
            boff[o] = off;
        }
        uint64_t *d_boff = nullptr;
        PLK_CUDA(cudaMallocAsync((void **)&d_boff, sizeof(uint64_t) * nb, s->stream));
        PLK_CUDA(cudaMemcpyAsync(d_boff, boff.data(), sizeof(uint64_t) * nb, cudaMemcpyHostToDevice, s->stream));
        const int grid = elem_grid(s, nb);
        k_marginal_gather<T><<<grid, kThreads, 0, s->stream>>>(sv, rb, d_boff, s->length >> m, nb, d_out);
        PLK_CHECK_LAUNCH();
        PLK_CUDA(cudaFreeAsync(d_boff, s->stream));
        PLK_CUDA(cudaStreamSynchronize(s->stream));
    }
    PLK_CUDA(cudaMemcpyAsync(out, d_out, sizeof(double) * nb, cudaMemcpyDeviceToHost, s->stream));
    PLK_CUDA(cudaFreeAsync(d_out, s->stream));
    PLK_CUDA(cudaStreamSynchronize(s->stream));
    return PLK_OK;
}

} // namespace plk

using namespace plk;

extern "C" {

PLK_API int plk_probs(plk_state s, const int64_t *wires, int32_t nw, double *out) {
    PLK_TRY(check_state(s));
    if (!out) PLK_FAIL(PLK_ERR_INVALID_ARG, "null output");
    PLK_TRY(check_wires(s, wires, nw));
    PLK_CUDA(cudaSetDevice(s->device));
    bool full = nw == 0;
    if (nw == s->nq) {
        full = true;
        for (int j = 0; j < nw; j++)
            if (wires[j] != j) full = false;
    }
    if (full) {
        double *d_p = nullptr;
        PLK_CUDA(cudaMallocAsync((void **)&d_p, sizeof(double) * s->length, s->stream));
        const int grid = elem_grid(s, s->length);
        if (s->dtype == PLK_C64) k_probs<float><<<grid, kThreads, 0, s->stream>>>((const float2 *)s->data, d_p, s->length);
        else k_probs<double><<<grid, kThreads, 0, s->stream>>>((const double2 *)s->data, d_p, s->length);
        PLK_CHECK_LAUNCH();
        PLK_CUDA(cudaMemcpyAsync(out, d_p, sizeof(double) * s->length, cudaMemcpyDeviceToHost, s->stream));
        PLK_CUDA(cudaFreeAsync(d_p, s->stream));
        PLK_CUDA(cudaStreamSynchronize(s->stream));
        return PLK_OK;
    }
    // Output order of the reference's probs(wires) (MeasuresKokkos.hpp:418-517):
    // marginals over the sorted wires, then transposed with
    // getTransposedIndexFunctor (MeasuresFunctors.hpp:162-182), which maps
    // output bit j to sorted position order[j] (order = argsort(wires)).
    // Output bit j therefore reads wire wires[order[order[j]]]; this equals
    // the requested order whenever the permutation is an involution.
    std::vector<int> order(nw);
    for (int j = 0; j < nw; j++) order[j] = j;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return wires[a] < wires[b]; });
    std::vector<int64_t> eff(nw);
    for (int j = 0; j < nw; j++) eff[j] = wires[order[order[j]]];
    return s->dtype == PLK_C64 ? marginal_impl<float>(s, eff.data(), nw, out)
                               : marginal_impl<double>(s, eff.data(), nw, out);
}

PLK_API int plk_cdf(plk_state s, double *out) {
    PLK_TRY(check_state(s));
    if (!out) PLK_FAIL(PLK_ERR_INVALID_ARG, "null output");
    PLK_CUDA(cudaSetDevice(s->device));
    double *d_cdf = nullptr;
    PLK_CUDA(cudaMallocAsync((void **)&d_cdf, sizeof(double) * s->length, s->stream));
    PLK_TRY(cdf_any(s, d_cdf));
    PLK_CUDA(cudaMemcpyAsync(out, d_cdf, sizeof(double) * s->length, cudaMemcpyDeviceToHost, s->stream));
    PLK_CUDA(cudaFreeAsync(d_cdf, s->stream));
    PLK_CUDA(cudaStreamSynchronize(s->stream));
    return PLK_OK;
}

PLK_API int plk_sample_from_uniforms(plk_state s, const double *uniforms, uint64_t shots, int64_t *out_bits) {
    PLK_TRY(check_state(s));
    if (shots == 0) return PLK_OK;
    if (!uniforms || !out_bits) PLK_FAIL(PLK_ERR_INVALID_ARG, "null argument");
    PLK_CUDA(cudaSetDevice(s->device));
    double *d_u = nullptr;
    PLK_CUDA(cudaMallocAsync((void **)&d_u, sizeof(double) * shots, s->stream));
    PLK_CUDA(cudaMemcpyAsync(d_u, uniforms, sizeof(double) * shots, cudaMemcpyHostToDevice, s->stream));
    int st = sample_with_uniforms_dev(s, d_u, shots, out_bits);
    cudaFreeAsync(d_u, s->stream);
    cudaStreamSynchronize(s->stream);
    return st;
}

PLK_API int plk_generate_samples(plk_state s, uint64_t shots, uint64_t seed, int64_t *out_bits) {
    PLK_TRY(check_state(s));
    if (shots == 0) return PLK_OK;
    if (!out_bits) PLK_FAIL(PLK_ERR_INVALID_ARG, "null output");
    PLK_CUDA(cudaSetDevice(s->device));
    double *d_u = nullptr;
    PLK_CUDA(cudaMallocAsync((void **)&d_u, sizeof(double) * shots, s->stream));
    const int grid = elem_grid(s, (shots + 1) / 2);
    k_philox_uniforms<<<grid, kThreads, 0, s->stream>>>(seed, shots, d_u);
    PLK_CHECK_LAUNCH();
    int st = sample_with_uniforms_dev(s, d_u, shots, out_bits);
    cudaFreeAsync(d_u, s->stream);
    cudaStreamSynchronize(s->stream);
    return st;
}

PLK_API int plk_search_cdf(const double *cdf, uint64_t length, int32_t nq, const double *uniforms, uint64_t shots,
                           int64_t *out_bits, int device) {
    if (!cdf || !uniforms || !out_bits) PLK_FAIL(PLK_ERR_INVALID_ARG, "null argument");
    if (nq < 1 || nq > 40 || length != (1ULL << nq)) PLK_FAIL(PLK_ERR_INVALID_ARG, "CDF length must be 2^num_qubits");
    if (shots == 0) return PLK_OK;
    DeviceCtx *d = nullptr;
    PLK_TRY(device_ctx(device, &d));
    PLK_CUDA(cudaSetDevice(device));
    cudaStream_t st = d->stream;
    double *d_cdf = nullptr, *d_u = nullptr;
    int64_t *d_bits = nullptr;
    PLK_CUDA(cudaMallocAsync((void **)&d_cdf, sizeof(double) * length, st));
    PLK_CUDA(cudaMallocAsync((void **)&d_u, sizeof(double) * shots, st));
    PLK_CUDA(cudaMallocAsync((void **)&d_bits, sizeof(int64_t) * shots * nq, st));
    PLK_CUDA(cudaMemcpyAsync(d_cdf, cdf, sizeof(double) * length, cudaMemcpyHostToDevice, st));
    PLK_CUDA(cudaMemcpyAsync(d_u, uniforms, sizeof(double) * shots, cudaMemcpyHostToDevice, st));
    const unsigned grid = (unsigned)std::min<uint64_t>((shots + kThreads - 1) / kThreads, (uint64_t)d->sm_count * 8);
    k_sample<<<std::max(1u, grid), kThreads, 0, st>>>(d_cdf, length, nq, d_u, shots, d_bits);
    PLK_CHECK_LAUNCH();
    PLK_CUDA(cudaMemcpyAsync(out_bits, d_bits, sizeof(int64_t) * shots * nq, cudaMemcpyDeviceToHost, st));
    PLK_CUDA(cudaFreeAsync(d_cdf, st));
    PLK_CUDA(cudaFreeAsync(d_u, st));
    PLK_CUDA(cudaFreeAsync(d_bits, st));
    PLK_CUDA(cudaStreamSynchronize(st));
    return PLK_OK;
}

} // extern "C"
