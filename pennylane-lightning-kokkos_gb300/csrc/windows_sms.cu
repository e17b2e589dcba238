// windows_sms.cu — complex64 register windows over one state (forward and
// backward), amplitudes staged in shared memory (k_state_window_sms in
// window_sms.cuh); launched by windows.cu.
#include <algorithm>
#include <atomic>

#include "window_sms.cuh"

namespace plk {

// CTAs of a complex64 window launch over `groups` 16-amplitude groups
int window_sms_grid(int sm_count, uint64_t groups, bool bwd) {
    const uint64_t want = (groups + kWinThreadsSms - 1) / kWinThreadsSms;
    const uint64_t cap = (uint64_t)sm_count * (bwd ? kSmsCtasBwd : kSmsCtasFwd);
    return (int)std::max<uint64_t>(1, std::min(want, cap));
}

template <bool BWD>
static void launch_sms(int grid, cudaStream_t st, float2 *lam, float2 *hl, int nq, const EWin *wins, int wi,
                       int ntrain, const EOp *ops, const float2 *mats, const ETrain *train, double *bpart) {
    // more than 48 KiB of dynamic shared memory (backward) needs an opt-in, once per device
    static std::atomic<unsigned long long> opted{0};
    int dev = 0;
    cudaGetDevice(&dev);
    const unsigned long long bit = 1ull << (dev & 63);
    if (!(opted.load() & bit)) {
        cudaFuncSetAttribute(k_state_window_sms<BWD>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)sms_smem_bytes(BWD));
        opted.fetch_or(bit);
    }
    k_state_window_sms<BWD><<<grid, kWinThreadsSms, sms_smem_bytes(BWD, ntrain), st>>>(lam, hl, nq, wins, wi, ops,
                                                                                      mats, train, bpart);
}

void launch_window_sms(bool bwd, int grid, cudaStream_t st, float2 *lam, float2 *hl, int nq, const EWin *wins, int wi,
                       int ntrain, const EOp *ops, const float2 *mats, const ETrain *train, double *bpart) {
    if (bwd) launch_sms<true>(grid, st, lam, hl, nq, wins, wi, ntrain, ops, mats, train, bpart);
    else launch_sms<false>(grid, st, lam, hl, nq, wins, wi, 0, ops, mats, train, bpart);
}

} // namespace plk
