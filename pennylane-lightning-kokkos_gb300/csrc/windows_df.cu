// windows_df.cu — complex128 register windows on the FP32 pipe.
//
// The kernels of windows.cu for complex128 states, kept in their own
// translation unit (they are large and compile in parallel with it).  Ops in
// double-float arithmetic: window_df.cuh.
#include "window_df.cuh"

namespace plk {

constexpr int kWinThreadsDf = 256;

// complex128 windows on the FP32 pipe (window_df.cuh).  Between windows of
// one sweep the states stay in double-float form in their own buffers (a
// {re.hi, re.lo, im.hi, im.lo} float4 has the size of a double2): the first
// window splits the doubles (in_df = 0), the last joins them back
// (out_df = 0), the ones between move raw pairs.
template <bool BWD, bool SLIM>
__global__ void __launch_bounds__(kWinThreadsDf, 1)
    k_state_window_df(double2 *lam, double2 *hl, int nq, const EWin *__restrict__ wins, int wi,
                      const EOp *__restrict__ ops, const float4 *__restrict__ mats, const ETrain *__restrict__ train,
                      double *__restrict__ bpart, int in_df, int out_df) {
    __shared__ float2 part[kMaxWinTrain * kWinThreadsDf];
    const EWin w = wins[wi];
    const int tid = threadIdx.x;
    if (BWD)
        for (int t = 0; t < w.ntrain; t++) part[t * kWinThreadsDf + tid] = make_float2(0.0f, 0.0f);
    const uint32_t nu = 1u << (nq - kWinBits);
    const uint32_t bb[4] = {1u << w.rb[0], 1u << w.rb[1], 1u << w.rb[2], 1u << w.rb[3]};
    const uint32_t tstep = gridDim.x * kWinThreadsDf;
    for (uint32_t u = blockIdx.x * kWinThreadsDf + tid; u < nu; u += tstep) {
        uint32_t base = u;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const uint32_t lo = base & (bb[i] - 1);
            base = ((base ^ lo) << 1) | lo;
        }
        CDF lv[kWinAmps], hv[kWinAmps];
#pragma unroll
        for (int j = 0; j < kWinAmps; j++) {
            const uint32_t idx = base | ((j & 1) ? bb[0] : 0) | ((j & 2) ? bb[1] : 0) | ((j & 4) ? bb[2] : 0) |
                                 ((j & 8) ? bb[3] : 0);
            if (in_df) {
                const float4 a = reinterpret_cast<const float4 *>(lam)[idx];
                lv[j] = {{a.x, a.y}, {a.z, a.w}};
                if (BWD) {
                    const float4 b = reinterpret_cast<const float4 *>(hl)[idx];
                    hv[j] = {{b.x, b.y}, {b.z, b.w}};
                } else {
                    hv[j] = cdf_zero();
                }
            } else {
                lv[j] = cdf_split(lam[idx]);
                hv[j] = BWD ? cdf_split(hl[idx]) : cdf_zero();
            }
        }
        for (int k = 0; k < w.nops; k++) {
            const EOp op = ops[w.op0 + k];
            DAcc acc, acc1;
            if (BWD && op.red != 0xff) {
                const float2 p = part[op.red * kWinThreadsDf + tid];
                acc.h = p.x;
                acc.l = p.y;
            }
            window_op_df<BWD, SLIM>(op, lv, hv, base, bb, mats, acc, acc1);
            if (BWD && op.red != 0xff) {
                df_add(acc1.h, acc1.l, acc.h, acc.l);
                part[op.red * kWinThreadsDf + tid] = make_float2(acc.h, acc.l);
            }
        }
#pragma unroll
        for (int j = 0; j < kWinAmps; j++) {
            const uint32_t idx = base | ((j & 1) ? bb[0] : 0) | ((j & 2) ? bb[1] : 0) | ((j & 4) ? bb[2] : 0) |
                                 ((j & 8) ? bb[3] : 0);
            if (out_df) {
                reinterpret_cast<float4 *>(lam)[idx] = make_float4(lv[j].re.hi, lv[j].re.lo, lv[j].im.hi, lv[j].im.lo);
                if (BWD)
                    reinterpret_cast<float4 *>(hl)[idx] =
                        make_float4(hv[j].re.hi, hv[j].re.lo, hv[j].im.hi, hv[j].im.lo);
            } else {
                lam[idx] = make_double2(df_join(lv[j].re.hi, lv[j].re.lo), df_join(lv[j].im.hi, lv[j].im.lo));
                if (BWD)
                    hl[idx] = make_double2(df_join(hv[j].re.hi, hv[j].re.lo), df_join(hv[j].im.hi, hv[j].im.lo));
            }
        }
    }
    if (BWD && w.ntrain > 0) {
        __syncthreads();
        const int lane = tid & 31, warp = tid >> 5;
        for (int t = warp; t < w.ntrain; t += kWinThreadsDf / 32) {
            EAcc<float> acc;
#pragma unroll
            for (int i = 0; i < kWinThreadsDf / 32; i++) {
                const float2 p = part[t * kWinThreadsDf + i * 32 + lane];
                df_add(p.x, p.y, acc.h, acc.l);
            }
            const double sum = acc.warp_sum();
            if (lane == 0) {
                const ETrain tr = train[w.tr0 + t];
                bpart[(size_t)tr.slot * gridDim.x + blockIdx.x] = (double)tr.gscale * sum;
            }
        }
    }
}


void launch_window_df(bool bwd, bool slim, int grid, cudaStream_t st, double2 *lam, double2 *hl, int nq,
                      const EWin *wins, int wi, const EOp *ops, const float4 *mats, const ETrain *train,
                      double *bpart, int in_df, int out_df) {
    // one kernel per direction: the slim variant (one-wire ops and CNOTs
    // only) measured no faster here, double-float work dominates
    (void)slim;
    if (bwd)
        k_state_window_df<true, false><<<grid, kWinThreadsDf, 0, st>>>(lam, hl, nq, wins, wi, ops, mats, train, bpart,
                                                                       in_df, out_df);
    else
        k_state_window_df<false, false><<<grid, kWinThreadsDf, 0, st>>>(lam, hl, nq, wins, wi, ops, mats, train,
                                                                        bpart, in_df, out_df);
}

} // namespace plk
