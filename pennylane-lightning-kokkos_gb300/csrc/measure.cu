// measure.cu — probabilities, CDF and sampling.
//
// Replaces MeasuresKokkos::probs / probs(wires) / generate_samples
// (simulator/MeasuresKokkos.hpp:389-569) and getProbFunctor, getCDFFunctor,
// Sampler, getSubProbFunctor and the transpose functors
// (simulator/MeasuresFunctors.hpp).
//
//  - probs(): |psi_k|^2 in double-float on the FP32 pipe, one FP64 add.
//  - probs(wires): marginals computed directly in the requested wire order
//    (no separate transpose pass): one warp per (bin, chunk of the bin's
//    amplitudes), chunks summed in order, so results are deterministic.
//  - CDF: exclusive scan over 4096-amplitude tiles in three one-pass
//    launches (tile masses, a one-block scan of the masses, per-tile scans).
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

// ------------------------------------------------------------ marginals --
// probs(wires): out[o] = sum of |psi_k|^2 over the amplitudes k whose
// measured bits spell o (output bit m-1-j is amplitude bit rev[j]).  The
// other n-m bits ("rest" bits) index the 2^(n-m) amplitudes of a bin.
// Work item (bin o, chunk c) is one warp: its lanes take consecutive rest
// indices, so when the lowest index bits are rest bits the warp reads
// consecutive amplitudes.  Items run with the bin index fastest, so warps
// that split a sector between bins run together.  Each lane accumulates in
// double-float, the warp reduces in FP64 in a fixed pattern, and chunks of a
// bin are summed in chunk order: the result does not depend on scheduling.
struct MargArgs {
    int rev[40];      // amplitude bit of output bit m-1-j
    int m;
    int rest_bit[40]; // rest bit positions, ascending
    int nrest_bits;
    int chunk_bits;   // log2 of the rest indices per chunk
    uint64_t lane_off[32]; // deposit of the lane index into the lowest rest bits
    uint64_t mid_mask;     // rest bits [5, chunk_bits) of the rest index
};

__device__ __forceinline__ uint64_t marg_bin_offset(const MargArgs &a, uint64_t o) {
    uint64_t off = 0;
    for (int j = 0; j < a.m; j++) off |= ((o >> (a.m - 1 - j)) & 1ULL) << a.rev[j];
    return off;
}

__device__ __forceinline__ uint64_t marg_deposit(const MargArgs &a, uint64_t r, int from_bit) {
    uint64_t d = 0;
    for (int j = from_bit; j < a.nrest_bits && (r >> j) != 0; j++) d |= ((r >> j) & 1ULL) << a.rest_bit[j];
    return d;
}

template <class T>
__global__ void __launch_bounds__(kThreads)
    k_marginal_warp(const c2_t<T> *__restrict__ sv, const MargArgs a, uint64_t nbins, uint64_t nitems,
                    double *__restrict__ dst) {
    const int lane = threadIdx.x & 31;
    const uint64_t wstep = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const uint64_t lane_off = a.lane_off[lane];
    for (uint64_t it = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; it < nitems; it += wstep) {
        const uint64_t o = it % nbins, c = it / nbins;
        const uint64_t base = marg_bin_offset(a, o) | marg_deposit(a, c << a.chunk_bits, a.chunk_bits) | lane_off;
        DAcc acc;
        // cur walks the subsets of mid_mask in increasing order (masked
        // increment: set the bits outside the mask, add one, clear them
        // again); it is back at zero after the last subset
        uint64_t cur = 0;
        do {
            // up to four loads in flight per lane
            uint64_t ad[4];
            int cnt = 0;
#pragma unroll
            for (int u = 0; u < 4; u++) {
                ad[u] = base | cur;
                cnt = u + 1;
                cur = ((cur | ~a.mid_mask) + 1) & a.mid_mask;
                if (cur == 0) break;
            }
            c2_t<T> v[4];
#pragma unroll
            for (int u = 0; u < 4; u++)
                if (u < cnt) v[u] = sv[ad[u]];
#pragma unroll
            for (int u = 0; u < 4; u++)
                if (u < cnt) acc.add(df_norm2(to_cdf(v[u])));
        } while (cur != 0);
        double s = acc.value();
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
        if (lane == 0) dst[it] = s;
    }
}

// fewer than 32 amplitudes per bin: one thread per bin
template <class T>
__global__ void __launch_bounds__(kThreads)
    k_marginal_thread(const c2_t<T> *__restrict__ sv, const MargArgs a, uint64_t nbins, uint64_t nrest,
                      double *__restrict__ out) {
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t o = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; o < nbins; o += step) {
        const uint64_t off = marg_bin_offset(a, o);
        DAcc acc;
        for (uint64_t r = 0; r < nrest; r++) acc.add(df_norm2(to_cdf(sv[off | marg_deposit(a, r, 0)])));
        out[o] = acc.value();
    }
}

// out[o] = sum over chunks c (in order) of part[c * nbins + o]
__global__ void k_marginal_chunks(const double *__restrict__ part, uint64_t nbins, int nchunks,
                                  double *__restrict__ out) {
    const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t o = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; o < nbins; o += step) {
        double s = 0.0;
        for (int c = 0; c < nchunks; c++) s += part[(uint64_t)c * nbins + o];
        out[o] = s;
    }
}

// ------------------------------------------------------------------ CDF --
// Exclusive prefix sum of |psi_k|^2 in three launches, each one pass:
//   k_cdf_tile_sums  - the mass of every 4096-amplitude tile (double-float
//                      per thread, FP64 across the block);
//   k_cdf_scan_tiles - one block scans the tile masses in FP64;
//   k_cdf_tiles      - every tile re-reads its amplitudes, stages |psi_k|^2
//                      (double-float) in shared memory, scans each thread's
//                      16 consecutive values and the block's thread totals in
//                      double-float, adds the tile offset and writes the
//                      doubles back through shared memory (coalesced).
// Values are within about 1e-14 of the exact prefix sums of a normalised
// state.
constexpr int kCdfPer = 16;
constexpr int kCdfTile = kThreads * kCdfPer; // 4096 amplitudes
constexpr int kCdfScanThreads = 1024;

// shared-memory slot of tile element e: one pad entry every 16 makes both
// the coalesced (e = j*256 + t) and the per-thread (e = 16t + j) patterns
// free of bank conflicts for 8-byte elements
__device__ __forceinline__ int cdf_slot(int e) { return e + (e >> 4); }

template <class T>
__global__ void __launch_bounds__(kThreads)
    k_cdf_tile_sums(const c2_t<T> *__restrict__ sv, uint64_t n, double *__restrict__ tile_sum) {
    __shared__ double wsum[kThreads / 32];
    const uint64_t base = (uint64_t)blockIdx.x * kCdfTile;
    // all sixteen loads in flight before the sums
    c2_t<T> v[kCdfPer];
#pragma unroll
    for (int j = 0; j < kCdfPer; j++) {
        const uint64_t k = base + (uint64_t)j * kThreads + threadIdx.x;
        v[j] = k < n ? sv[k] : mk<c2_t<T>>(0, 0);
    }
    DAcc acc;
#pragma unroll
    for (int j = 0; j < kCdfPer; j++) acc.add(df_norm2(to_cdf(v[j])));
    double s = acc.value();
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < kThreads / 32; w++) t += wsum[w];
        tile_sum[blockIdx.x] = t;
    }
}

// in-place exclusive scan of ntiles doubles by one block of kCdfScanThreads
__global__ void __launch_bounds__(kCdfScanThreads) k_cdf_scan_tiles(double *__restrict__ v, uint64_t ntiles) {
    __shared__ double wtot[kCdfScanThreads / 32];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const uint64_t chunk = (ntiles + kCdfScanThreads - 1) / kCdfScanThreads;
    const uint64_t lo = (uint64_t)t * chunk, hi = lo + chunk < ntiles ? lo + chunk : ntiles;
    double tot = 0.0;
    for (uint64_t i = lo; i < hi; i++) tot += v[i];
    // inclusive warp scan of the thread totals
    double inc = tot;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const double y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) wtot[w] = inc;
    __syncthreads();
    double excl = __shfl_up_sync(0xffffffffu, inc, 1);
    if (lane == 0) excl = 0.0;
    double run = 0.0;
    for (int j = 0; j < w; j++) run += wtot[j];
    run += excl;
    for (uint64_t i = lo; i < hi; i++) {
        const double x = v[i];
        v[i] = run;
        run += x;
    }
}

template <class T>
__global__ void __launch_bounds__(kThreads)
    k_cdf_tiles(const c2_t<T> *__restrict__ sv, uint64_t n, const double *__restrict__ tile_off,
                double *__restrict__ cdf) {
    __shared__ __align__(16) float2 stage[kCdfTile + kCdfTile / 16];
    __shared__ float2 wtot[kThreads / 32];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const uint64_t base = (uint64_t)blockIdx.x * kCdfTile;
    // 1. coalesced loads (all sixteen in flight), |psi|^2 as double-float
    // into shared memory
    {
        c2_t<T> v[kCdfPer];
#pragma unroll
        for (int j = 0; j < kCdfPer; j++) {
            const uint64_t k = base + (uint64_t)j * kThreads + t;
            v[j] = k < n ? sv[k] : mk<c2_t<T>>(0, 0);
        }
#pragma unroll
        for (int j = 0; j < kCdfPer; j++) {
            const DF p = df_norm2(to_cdf(v[j]));
            stage[cdf_slot(j * kThreads + t)] = make_float2(p.hi, p.lo);
        }
    }
    __syncthreads();
    // 2. this thread's 16 consecutive values and their sum
    DF p[kCdfPer];
    float th = 0.0f, tl = 0.0f;
#pragma unroll
    for (int j = 0; j < kCdfPer; j++) {
        const float2 q = stage[cdf_slot(t * kCdfPer + j)];
        p[j] = {q.x, q.y};
        df_add(q.x, q.y, th, tl);
    }
    // 3. exclusive scan of the thread sums across the block (double-float)
    float ih = th, il = tl;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const float yh = __shfl_up_sync(0xffffffffu, ih, o), yl = __shfl_up_sync(0xffffffffu, il, o);
        if (lane >= o) df_add(yh, yl, ih, il);
    }
    if (lane == 31) wtot[w] = make_float2(ih, il);
    float eh = __shfl_up_sync(0xffffffffu, ih, 1), el = __shfl_up_sync(0xffffffffu, il, 1);
    if (lane == 0) eh = el = 0.0f;
    __syncthreads();
    // running value: tile offset + earlier warps + earlier lanes
    float rh, rl;
    {
        const double off = tile_off[blockIdx.x];
        const float oh = (float)off;
        rh = oh;
        rl = (float)(off - (double)oh);
    }
    for (int j = 0; j < w; j++) df_add(wtot[j].x, wtot[j].y, rh, rl);
    df_add(eh, el, rh, rl);
    // 4. the prefixes, staged as doubles in the same buffer, then coalesced stores
    double *outst = reinterpret_cast<double *>(stage);
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kCdfPer; j++) {
        outst[cdf_slot(t * kCdfPer + j)] = df_result(rh, rl);
        df_add(p[j].hi, p[j].lo, rh, rl);
    }
    __syncthreads();
#pragma unroll 4
    for (int j = 0; j < kCdfPer; j++) {
        const int e = j * kThreads + t;
        const uint64_t k = base + e;
        if (k < n) cdf[k] = outst[cdf_slot(e)];
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
// ------------------------------------------------------------- helpers --
template <class T> static int cdf_device(plk_state s, double *d_cdf) {
    const uint64_t n = s->length;
    const uint64_t ntiles = (n + kCdfTile - 1) / kCdfTile;
    double *d_tiles = nullptr;
    PoolBuf d_tiles_buf(s->stream);
    PLK_TRY(pool_alloc(s->device, &d_tiles_buf.p, sizeof(double) * ntiles, s->stream));
    d_tiles = d_tiles_buf.as<double>();
    auto *sv = (const c2_t<T> *)s->data;
    k_cdf_tile_sums<T><<<(unsigned)ntiles, kThreads, 0, s->stream>>>(sv, n, d_tiles);
    PLK_CHECK_LAUNCH();
    k_cdf_scan_tiles<<<1, kCdfScanThreads, 0, s->stream>>>(d_tiles, ntiles);
    PLK_CHECK_LAUNCH();
    k_cdf_tiles<T><<<(unsigned)ntiles, kThreads, 0, s->stream>>>(sv, n, d_tiles, d_cdf);
    PLK_CHECK_LAUNCH();
    return PLK_OK;
}


static int cdf_any(plk_state s, double *d_cdf) {
    return s->dtype == PLK_C64 ? cdf_device<float>(s, d_cdf) : cdf_device<double>(s, d_cdf);
}

static int sample_with_uniforms_dev(plk_state s, const double *d_u, uint64_t shots, int64_t *out_bits) {
    double *d_cdf = nullptr;
    int64_t *d_bits = nullptr;
    PoolBuf d_cdf_buf(s->stream);
    PLK_TRY(pool_alloc(s->device, &d_cdf_buf.p, sizeof(double) * s->length, s->stream));
    d_cdf = d_cdf_buf.as<double>();
    PLK_TRY(cdf_any(s, d_cdf));
    PoolBuf d_bits_buf(s->stream);
    PLK_TRY(pool_alloc(s->device, &d_bits_buf.p, sizeof(int64_t) * shots * s->nq, s->stream));
    d_bits = d_bits_buf.as<int64_t>();
    const int grid = elem_grid(s, shots);
    k_sample<<<grid, kThreads, 0, s->stream>>>(d_cdf, s->length, s->nq, d_u, shots, d_bits);
    PLK_CHECK_LAUNCH();
    PLK_CUDA(cudaMemcpyAsync(out_bits, d_bits, sizeof(int64_t) * shots * s->nq, cudaMemcpyDeviceToHost, s->stream));
    PLK_CUDA(cudaStreamSynchronize(s->stream));
    return PLK_OK;
}

template <class T> static int marginal_impl(plk_state s, const int64_t *wires, int m, double *out) {
    MargArgs a;
    std::memset(&a, 0, sizeof(a));
    a.m = m;
    uint64_t measured = 0;
    for (int j = 0; j < m; j++) {
        a.rev[j] = s->nq - 1 - (int)wires[j];
        measured |= 1ULL << a.rev[j];
    }
    for (int b = 0; b < s->nq; b++)
        if (!((measured >> b) & 1)) a.rest_bit[a.nrest_bits++] = b;
    const uint64_t nb = 1ULL << m;
    const uint64_t nrest = 1ULL << a.nrest_bits;
    auto *sv = (const c2_t<T> *)s->data;
    DeviceCtx *d = nullptr;
    PLK_TRY(device_ctx(s->device, &d));
    double *d_out = nullptr;
    PoolBuf d_out_buf(s->stream);
    PLK_TRY(pool_alloc(s->device, &d_out_buf.p, sizeof(double) * nb, s->stream));
    d_out = d_out_buf.as<double>();
    if (nrest < 32) {
        k_marginal_thread<T><<<elem_grid(s, nb), kThreads, 0, s->stream>>>(sv, a, nb, nrest, d_out);
        PLK_CHECK_LAUNCH();
    } else {
        // chunks per bin: enough warps to fill the device twice over, at
        // least 32 rest indices (one per lane) per chunk
        const uint64_t want_warps = (uint64_t)d->sm_count * (d->max_threads_per_sm / 32) * 2;
        int cb = 0;
        while (((nb << cb) < want_warps) && (a.nrest_bits - (cb + 1) >= 5)) cb++;
        a.chunk_bits = a.nrest_bits - cb;
        for (int l = 0; l < 32; l++) {
            uint64_t dep = 0;
            for (int j = 0; j < 5; j++)
                if ((l >> j) & 1) dep |= 1ULL << a.rest_bit[j];
            a.lane_off[l] = dep;
        }
        a.mid_mask = 0;
        for (int j = 5; j < a.chunk_bits; j++) a.mid_mask |= 1ULL << a.rest_bit[j];
        const uint64_t nchunks = 1ULL << cb;
        const uint64_t nitems = nb * nchunks;
        const uint64_t grid64 = std::min<uint64_t>((nitems * 32 + kThreads - 1) / kThreads,
                                                   (uint64_t)d->sm_count * (d->max_threads_per_sm / kThreads) * 4);
        const unsigned grid = (unsigned)std::max<uint64_t>(1, grid64);
        if (nchunks == 1) {
            k_marginal_warp<T><<<grid, kThreads, 0, s->stream>>>(sv, a, nb, nitems, d_out);
            PLK_CHECK_LAUNCH();
        } else {
            double *d_part = nullptr;
            PoolBuf d_part_buf(s->stream);
            PLK_TRY(pool_alloc(s->device, &d_part_buf.p, sizeof(double) * nitems, s->stream));
            d_part = d_part_buf.as<double>();
            k_marginal_warp<T><<<grid, kThreads, 0, s->stream>>>(sv, a, nb, nitems, d_part);
            PLK_CHECK_LAUNCH();
            k_marginal_chunks<<<elem_grid(s, nb), kThreads, 0, s->stream>>>(d_part, nb, (int)nchunks, d_out);
            PLK_CHECK_LAUNCH();
        }
    }
    PLK_CUDA(cudaMemcpyAsync(out, d_out, sizeof(double) * nb, cudaMemcpyDeviceToHost, s->stream));
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
        PoolBuf d_p_buf(s->stream);
        PLK_TRY(pool_alloc(s->device, &d_p_buf.p, sizeof(double) * s->length, s->stream));
        d_p = d_p_buf.as<double>();
        const int grid = elem_grid(s, s->length);
        if (s->dtype == PLK_C64) k_probs<float><<<grid, kThreads, 0, s->stream>>>((const float2 *)s->data, d_p, s->length);
        else k_probs<double><<<grid, kThreads, 0, s->stream>>>((const double2 *)s->data, d_p, s->length);
        PLK_CHECK_LAUNCH();
        PLK_CUDA(cudaMemcpyAsync(out, d_p, sizeof(double) * s->length, cudaMemcpyDeviceToHost, s->stream));
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
    PoolBuf d_cdf_buf(s->stream);
    PLK_TRY(pool_alloc(s->device, &d_cdf_buf.p, sizeof(double) * s->length, s->stream));
    d_cdf = d_cdf_buf.as<double>();
    PLK_TRY(cdf_any(s, d_cdf));
    PLK_CUDA(cudaMemcpyAsync(out, d_cdf, sizeof(double) * s->length, cudaMemcpyDeviceToHost, s->stream));
    PLK_CUDA(cudaStreamSynchronize(s->stream));
    return PLK_OK;
}

PLK_API int plk_sample_from_uniforms(plk_state s, const double *uniforms, uint64_t shots, int64_t *out_bits) {
    PLK_TRY(check_state(s));
    if (shots == 0) return PLK_OK;
    if (!uniforms || !out_bits) PLK_FAIL(PLK_ERR_INVALID_ARG, "null argument");
    PLK_CUDA(cudaSetDevice(s->device));
    double *d_u = nullptr;
    PoolBuf d_u_buf(s->stream);
    PLK_TRY(pool_alloc(s->device, &d_u_buf.p, sizeof(double) * shots, s->stream));
    d_u = d_u_buf.as<double>();
    PLK_CUDA(cudaMemcpyAsync(d_u, uniforms, sizeof(double) * shots, cudaMemcpyHostToDevice, s->stream));
    int st = sample_with_uniforms_dev(s, d_u, shots, out_bits);
    cudaStreamSynchronize(s->stream);
    return st;
}

PLK_API int plk_generate_samples(plk_state s, uint64_t shots, uint64_t seed, int64_t *out_bits) {
    PLK_TRY(check_state(s));
    if (shots == 0) return PLK_OK;
    if (!out_bits) PLK_FAIL(PLK_ERR_INVALID_ARG, "null output");
    PLK_CUDA(cudaSetDevice(s->device));
    double *d_u = nullptr;
    PoolBuf d_u_buf(s->stream);
    PLK_TRY(pool_alloc(s->device, &d_u_buf.p, sizeof(double) * shots, s->stream));
    d_u = d_u_buf.as<double>();
    const int grid = elem_grid(s, (shots + 1) / 2);
    k_philox_uniforms<<<grid, kThreads, 0, s->stream>>>(seed, shots, d_u);
    PLK_CHECK_LAUNCH();
    int st = sample_with_uniforms_dev(s, d_u, shots, out_bits);
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
    PoolBuf d_cdf_buf(st);
    PLK_TRY(pool_alloc(device, &d_cdf_buf.p, sizeof(double) * length, st));
    d_cdf = d_cdf_buf.as<double>();
    PoolBuf d_u_buf(st);
    PLK_TRY(pool_alloc(device, &d_u_buf.p, sizeof(double) * shots, st));
    d_u = d_u_buf.as<double>();
    PoolBuf d_bits_buf(st);
    PLK_TRY(pool_alloc(device, &d_bits_buf.p, sizeof(int64_t) * shots * nq, st));
    d_bits = d_bits_buf.as<int64_t>();
    PLK_CUDA(cudaMemcpyAsync(d_cdf, cdf, sizeof(double) * length, cudaMemcpyHostToDevice, st));
    PLK_CUDA(cudaMemcpyAsync(d_u, uniforms, sizeof(double) * shots, cudaMemcpyHostToDevice, st));
    const unsigned grid = (unsigned)std::min<uint64_t>((shots + kThreads - 1) / kThreads, (uint64_t)d->sm_count * 8);
    k_sample<<<std::max(1u, grid), kThreads, 0, st>>>(d_cdf, length, nq, d_u, shots, d_bits);
    PLK_CHECK_LAUNCH();
    PLK_CUDA(cudaMemcpyAsync(out_bits, d_bits, sizeof(int64_t) * shots * nq, cudaMemcpyDeviceToHost, st));
    PLK_CUDA(cudaStreamSynchronize(st));
    return PLK_OK;
}

} // extern "C"
