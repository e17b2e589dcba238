// windows_df.cu — complex128 register windows on the FP32 pipe, forward
// sweep.
//
// The kernels of windows.cu for complex128 states (k_state_window_df in
// window_df.cuh), one translation unit per direction so that they compile in
// parallel (windows_df.cu holds the backward one).
#include "window_df.cuh"

namespace plk {

void launch_window_df_fwd(int grid, cudaStream_t st, double2 *lam, double2 *hl, int nq, const EWin *wins, int wi,
                          const EOp *ops, const float4 *mats, const ETrain *train, double *bpart, int in_df,
                          int out_df) {
    k_state_window_df<false, false><<<grid, kWinThreadsDf, 0, st>>>(lam, hl, nq, wins, wi, ops, mats, train, bpart,
                                                                   in_df, out_df);
}

} // namespace plk
