// dense_tc.cu — complex64 dense matrices on 5 or 6 wires on the tensor cores.
//
// applyMultiQubitOp (StateVectorKokkos.hpp:757-796, multiQubitOpFunctor,
// GateFunctors.hpp:195-300) for a D x D matrix, D = 2^K: every group of D
// amplitudes (the amplitudes that differ only in the K target bits) is
// multiplied by U.  As a real GEMM over a tile of 16 groups:
//   Y (16 x 2D) = X (16 x 2D) W (2D x 2D),  X = [Re v | Im v],
//   W = [[Re U^T, Im U^T], [-Im U^T, Re U^T]],  Y = [Re Uv | Im Uv].
// Each warp runs mma.sync m16n8k8 with TF32 operands; FP32 accuracy comes
// from three products per step, x_hi w_hi + x_hi w_lo + x_lo w_hi, where
// a_hi is a rounded to TF32 (10 mantissa bits) and a_lo = a - a_hi rounded
// again (the dropped x_lo w_lo term is below 2^-22 of the product).  W's two
// parts are built on the host and staged in shared memory; a warp gathers its
// 16 groups into shared memory (lanes over groups, so a warp reads
// consecutive amplitudes when the target bits are not the lowest), runs the
// MMAs with accumulators in registers, and writes the outputs back through
// the same shared tile.
#include <atomic>
#include <cstring>
#include <vector>

#include "plk_internal.cuh"

namespace plk {

constexpr int kTcWarps = 8;

static std::atomic<int> g_dense_tc{1};
bool dense_tc_enabled() { return g_dense_tc.load(std::memory_order_relaxed) != 0; }

__device__ __forceinline__ uint32_t to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ void mma_tf32(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, "
                 "{%8, %9}, {%0, %1, %2, %3};"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Shared memory: W hi and lo ([2D][2D] floats each, row = reduction index,
// row stride 2D + 8 floats), then per warp an X tile of 16 rows x 2D floats
// (row stride 2D + 4 floats): the strides put the fragment loads of one warp
// on distinct banks.
template <int K> __host__ __device__ constexpr size_t tc_smem_bytes() {
    constexpr int N2 = 2 << K;
    return sizeof(float) * ((size_t)2 * N2 * (N2 + 8) + (size_t)kTcWarps * 16 * (N2 + 4));
}

template <int K>
__global__ void __launch_bounds__(kTcWarps * 32)
    k_dense_tc(float2 *__restrict__ sv, const float *__restrict__ w_hi, const float *__restrict__ w_lo,
               const uint64_t *__restrict__ off, Masks gm, uint64_t ngroups) {
    constexpr int D = 1 << K, N2 = 2 * D, XS = N2 + 4, WS = N2 + 8, NT = N2 / 8, KT = N2 / 8;
    extern __shared__ __align__(16) float tc_smem[];
    float *Wh = tc_smem, *Wl = Wh + N2 * WS;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float *X = Wl + N2 * WS + warp * 16 * XS;
    for (int i = threadIdx.x; i < N2 * N2; i += blockDim.x) {
        Wh[(i / N2) * WS + i % N2] = w_hi[i];
        Wl[(i / N2) * WS + i % N2] = w_lo[i];
    }
    __syncthreads();
    const int gid = lane >> 2, tig = lane & 3;
    const int g_mine = lane & 15, c_first = lane >> 4; // gather / scatter: lane -> (group, first amplitude)
    const uint64_t tiles = (ngroups + 15) / 16;
    for (uint64_t tile = (uint64_t)blockIdx.x * kTcWarps + warp; tile < tiles;
         tile += (uint64_t)gridDim.x * kTcWarps) {
        const uint64_t g = tile * 16 + g_mine;
        const bool valid = g < ngroups;
        uint64_t base = g & gm.m[0];
#pragma unroll
        for (int j = 1; j <= K; j++) base |= (g << j) & gm.m[j];
        // gather: X[row][c] = Re v_c, X[row][D + c] = Im v_c
        for (int c = c_first; c < D; c += 2) {
            const float2 v = valid ? sv[base + off[c]] : make_float2(0.0f, 0.0f);
            X[g_mine * XS + c] = v.x;
            X[g_mine * XS + D + c] = v.y;
        }
        __syncwarp();
        float acc[NT][4];
#pragma unroll
        for (int n = 0; n < NT; n++) acc[n][0] = acc[n][1] = acc[n][2] = acc[n][3] = 0.0f;
#pragma unroll 1
        for (int kt = 0; kt < KT; kt++) {
            const int k0 = kt * 8;
            const float xa[4] = {X[gid * XS + k0 + tig], X[(gid + 8) * XS + k0 + tig], X[gid * XS + k0 + tig + 4],
                                 X[(gid + 8) * XS + k0 + tig + 4]};
            uint32_t ah[4], al[4];
#pragma unroll
            for (int i = 0; i < 4; i++) {
                ah[i] = to_tf32(xa[i]);
                al[i] = to_tf32(xa[i] - __uint_as_float(ah[i]));
            }
#pragma unroll
            for (int n = 0; n < NT; n++) {
                const int col = n * 8 + gid;
                const uint32_t bh0 = __float_as_uint(Wh[(k0 + tig) * WS + col]);
                const uint32_t bh1 = __float_as_uint(Wh[(k0 + tig + 4) * WS + col]);
                const uint32_t bl0 = __float_as_uint(Wl[(k0 + tig) * WS + col]);
                const uint32_t bl1 = __float_as_uint(Wl[(k0 + tig + 4) * WS + col]);
                mma_tf32(acc[n], al, bh0, bh1);
                mma_tf32(acc[n], ah, bl0, bl1);
                mma_tf32(acc[n], ah, bh0, bh1);
            }
        }
        __syncwarp();
        // accumulators -> X tile (row gid / gid + 8, columns 8n + 2 tig + {0, 1})
#pragma unroll
        for (int n = 0; n < NT; n++) {
            const int col = n * 8 + 2 * tig;
            X[gid * XS + col] = acc[n][0];
            X[gid * XS + col + 1] = acc[n][1];
            X[(gid + 8) * XS + col] = acc[n][2];
            X[(gid + 8) * XS + col + 1] = acc[n][3];
        }
        __syncwarp();
        if (valid)
            for (int c = c_first; c < D; c += 2) sv[base + off[c]] = make_float2(X[g_mine * XS + c], X[g_mine * XS + D + c]);
        __syncwarp();
    }
}

// U: D x D complex64, row-major (the matrix to apply, adjoint already taken).
int launch_dense_tc(plk_state s, const float2 *U, const uint64_t *hoff, const Masks &gm, int K) {
    if (K != 5 && K != 6) PLK_FAIL(PLK_ERR_UNSUPPORTED, "internal: tensor-core dense path takes 5 or 6 wires");
    const int D = 1 << K, N2 = 2 * D;
    // W = [[Re U^T, Im U^T], [-Im U^T, Re U^T]] split into TF32 hi and lo
    std::vector<float> wh((size_t)N2 * N2), wl((size_t)N2 * N2);
    auto tf32 = [](float x) { // round to nearest, ties away, 10 mantissa bits (the device's cvt.rna)
        uint32_t u;
        std::memcpy(&u, &x, 4);
        u = (u + 0x1000u) & 0xffffe000u;
        float r;
        std::memcpy(&r, &u, 4);
        return r;
    };
    for (int c = 0; c < D; c++)
        for (int r = 0; r < D; r++) {
            const float re = U[(size_t)r * D + c].x, im = U[(size_t)r * D + c].y;
            const float w[4] = {re, im, -im, re}; // [c][r], [c][D + r], [D + c][r], [D + c][D + r]
            const size_t idx[4] = {(size_t)c * N2 + r, (size_t)c * N2 + D + r, (size_t)(D + c) * N2 + r,
                                   (size_t)(D + c) * N2 + D + r};
            for (int q = 0; q < 4; q++) {
                const float h = tf32(w[q]);
                wh[idx[q]] = h;
                wl[idx[q]] = tf32(w[q] - h);
            }
        }
    const size_t wbytes = sizeof(float) * N2 * N2;
    char *buf = nullptr;
    const size_t total = 2 * wbytes + sizeof(uint64_t) * D;
    PLK_TRY(pool_alloc(s->device, (void **)&buf, total, s->stream));
    cudaError_t e = cudaMemcpyAsync(buf, wh.data(), wbytes, cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(buf + wbytes, wl.data(), wbytes, cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(buf + 2 * wbytes, hoff, sizeof(uint64_t) * D, cudaMemcpyHostToDevice, s->stream);
    const uint64_t ngroups = s->length >> K;
    DeviceCtx *d = nullptr;
    if (e == cudaSuccess && device_ctx(s->device, &d) == PLK_OK) {
        const uint64_t tiles = (ngroups + 15) / 16;
        const size_t smem = K == 5 ? tc_smem_bytes<5>() : tc_smem_bytes<6>();
        const int per_sm = K == 5 ? 3 : 1; // shared memory: 72 KB (K = 5), 207 KB (K = 6) per CTA
        const uint64_t want = (tiles + kTcWarps - 1) / kTcWarps;
        const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>(want, (uint64_t)d->sm_count * per_sm));
        const float *wh_d = (const float *)buf, *wl_d = (const float *)(buf + wbytes);
        const uint64_t *off_d = (const uint64_t *)(buf + 2 * wbytes);
        if (K == 5) {
            e = cudaFuncSetAttribute(k_dense_tc<5>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e == cudaSuccess)
                k_dense_tc<5><<<grid, kTcWarps * 32, smem, s->stream>>>((float2 *)s->data, wh_d, wl_d, off_d, gm, ngroups);
        } else {
            e = cudaFuncSetAttribute(k_dense_tc<6>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e == cudaSuccess)
                k_dense_tc<6><<<grid, kTcWarps * 32, smem, s->stream>>>((float2 *)s->data, wh_d, wl_d, off_d, gm, ngroups);
        }
        if (e == cudaSuccess) e = cudaGetLastError();
    }
    pool_free(buf, s->stream);
    // the host staging vectors are released on return: make the copies finish
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) PLK_FAIL(PLK_ERR_CUDA, std::string("tensor-core dense kernel: ") + cudaGetErrorString(e));
    return PLK_OK;
}

} // namespace plk

extern "C" {

PLK_API int plk_set_dense_tensor_cores(int32_t enable) {
    plk::g_dense_tc.store(enable != 0);
    return PLK_OK;
}

PLK_API int plk_get_dense_tensor_cores(int32_t *enabled) {
    if (!enabled) PLK_FAIL(PLK_ERR_INVALID_ARG, "null argument");
    *enabled = plk::g_dense_tc.load();
    return PLK_OK;
}

} // extern "C"
