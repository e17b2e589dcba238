// reduce.cuh — deterministic FP64 block reductions.
//
// Every reduction kernel accumulates FP64 partials per thread, reduces them
// across the block with warp shuffles in a fixed pattern, writes one partial
// per block, and the last block to finish (atomic ticket) sums the per-block
// partials in block order.  The grid is a function of the device and the
// problem size only, so a rerun gives the same bits; one launch per
// reduction, no host round trip until the caller reads the result.
#pragma once

#include "plk_internal.cuh"

namespace plk {

template <int NV>
__device__ __forceinline__ void block_reduce_finish(double (&acc)[NV], double *__restrict__ partials,
                                                    double *__restrict__ result, unsigned int *counter,
                                                    double post_scale = 1.0, int nvalid = NV) {
    __shared__ double sh[NV][kThreads / 32];
    __shared__ bool is_last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nblocks = gridDim.x;
#pragma unroll
    for (int v = 0; v < NV; v++) {
        double a = acc[v];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        if (lane == 0) sh[v][warp] = a;
    }
    __syncthreads();
    for (int v = threadIdx.x; v < NV; v += blockDim.x) {
        double s = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += sh[v][w];
        partials[(size_t)v * nblocks + blockIdx.x] = s;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) is_last = (atomicAdd(counter, 1u) == (unsigned)(nblocks - 1));
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    for (int v = warp; v < NV; v += (blockDim.x >> 5)) {
        double s = 0.0;
        for (int b = lane; b < nblocks; b += 32) s += __ldcg(partials + (size_t)v * nblocks + b);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0 && v < nvalid) result[v] = s * post_scale;
    }
    if (threadIdx.x == 0) *counter = 0u;
}

// Only the first `nvalid` results are written (NV may be a rounded-up
// template size).

// Copy `nv` reduced values to the host (pinned staging), synchronizing the
// state's stream.
int fetch_results(plk_state s, int nv, double *out);

} // namespace plk
