// windows_df_fwd.cu — complex128 register windows on the FP32 pipe, forward
// sweep.
//
// The kernel of windows.cu for complex128 states (k_state_window_dfs in
// window_dfs.cuh), one translation unit per direction so that they compile in
// parallel (windows_df.cu holds the backward one).
#include <atomic>

#include "window_dfs.cuh"

namespace plk {

void launch_window_df_fwd(int grid, cudaStream_t st, double2 *lam, double2 *hl, int nq, const EWin *wins, int wi,
                          const EOp *ops, const float4 *mats, const ETrain *train, double *bpart, int in_df,
                          int out_df) {
    // more than 48 KiB of dynamic shared memory needs an opt-in, once per device
    static std::atomic<unsigned long long> opted{0};
    int dev = 0;
    cudaGetDevice(&dev);
    const unsigned long long bit = 1ull << (dev & 63);
    if (!(opted.load() & bit)) {
        cudaFuncSetAttribute(k_state_window_dfs<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)dfs_smem_bytes(false));
        opted.fetch_or(bit);
    }
    k_state_window_dfs<false><<<grid, kWinThreadsDfs, dfs_smem_bytes(false), st>>>(lam, hl, nq, wins, wi, ops, mats,
                                                                                   train, bpart, in_df, out_df);
}

} // namespace plk
