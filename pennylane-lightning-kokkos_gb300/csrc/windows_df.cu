// windows_df.cu — complex128 register windows on the FP32 pipe, backward
// sweep (lambda and H lambda).
//
// The kernel of windows.cu for complex128 states (k_state_window_dfs in
// window_dfs.cuh), one translation unit per direction so that they compile in
// parallel (windows_df_fwd.cu holds the forward one).
#include <algorithm>
#include <atomic>

#include "window_dfs.cuh"

namespace plk {

// CTAs of a complex128 window launch over `groups` 16-amplitude groups
int window_df_grid(int sm_count, uint64_t groups, bool bwd) {
    const uint64_t want = (groups + kWinThreadsDfs - 1) / kWinThreadsDfs;
    const uint64_t cap = (uint64_t)sm_count * (bwd ? kDfsCtasBwd : kDfsCtasFwd);
    return (int)std::max<uint64_t>(1, std::min(want, cap));
}

void launch_window_df_bwd(int grid, cudaStream_t st, double2 *lam, double2 *hl, int nq, const EWin *wins, int wi,
                          int ntrain, const EOp *ops, const float4 *mats, const ETrain *train, double *bpart,
                          int in_df, int out_df) {
    // more than 48 KiB of dynamic shared memory needs an opt-in, once per device
    static std::atomic<unsigned long long> opted{0};
    int dev = 0;
    cudaGetDevice(&dev);
    const unsigned long long bit = 1ull << (dev & 63);
    if (!(opted.load() & bit)) {
        cudaFuncSetAttribute(k_state_window_dfs<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)dfs_smem_bytes(true));
        opted.fetch_or(bit);
    }
    k_state_window_dfs<true><<<grid, kWinThreadsDfs, dfs_smem_bytes(true, ntrain), st>>>(
        lam, hl, nq, wins, wi, ops, mats, train, bpart, in_df, out_df);
}

} // namespace plk
