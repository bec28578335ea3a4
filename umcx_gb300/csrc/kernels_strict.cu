// kernels_strict.cu - instances of the propagation kernel that evaluate every expression like the reference
// (IEEE division and square root, expf/logf/sinf/cosf/acosf).  This translation unit is compiled with
// --fmad=false so that no multiply-add is contracted, which keeps per-photon trajectories close to the CPU
// reference's for trajectory-level comparisons.
#include "launch.h"

namespace umcx_dev {

template <bool R, bool D>
static void launch_one(const LaunchChoice& lc, const KParams& P, const KBuffers& B, cudaStream_t st) {
    if (lc.rep == kRepWhole) k_forward<true, R, D, kRepWhole><<<lc.grid, lc.block, lc.smem, st>>>(P, B);
    else if (lc.rep == kRepPrefix) k_forward<true, R, D, kRepPrefix><<<lc.grid, lc.block, lc.smem, st>>>(P, B);
    else if (lc.rep == kRepOff) k_forward<true, R, D, kRepOff><<<lc.grid, lc.block, lc.smem, st>>>(P, B);
    else k_forward<true, R, D><<<lc.grid, lc.block, lc.smem, st>>>(P, B);
}

template <bool R, bool D>
static cudaError_t allow_big_smem() {
    cudaError_t e = allow_max_dynamic_smem(k_forward<true, R, D>);
    if (e == cudaSuccess) e = allow_max_dynamic_smem(k_forward<true, R, D, kRepPrefix>);
    if (e == cudaSuccess) e = allow_max_dynamic_smem(k_forward<true, R, D, kRepOff>);
    return e == cudaSuccess ? allow_max_dynamic_smem(k_forward<true, R, D, kRepWhole>) : e;
}
cudaError_t configure_strict_kernels() {
    cudaError_t e = allow_big_smem<false, false>();
    if (e == cudaSuccess) e = allow_big_smem<false, true>();
    if (e == cudaSuccess) e = allow_big_smem<true, false>();
    if (e == cudaSuccess) e = allow_big_smem<true, true>();
    return e;
}

void launch_forward_strict(const LaunchChoice& lc, const KParams& P, const KBuffers& B, cudaStream_t st) {
    if (lc.reflect) {
        if (lc.savedet) launch_one<true, true>(lc, P, B, st);
        else launch_one<true, false>(lc, P, B, st);
    } else {
        if (lc.savedet) launch_one<false, true>(lc, P, B, st);
        else launch_one<false, false>(lc, P, B, st);
    }
}

template <bool R, bool D>
static int occ_one(int block, size_t smem) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_forward<true, R, D>, block, smem) != cudaSuccess) return 0;
    return n;
}

int occupancy_strict(bool reflect, bool savedet, int block, size_t smem) {
    if (reflect) return savedet ? occ_one<true, true>(block, smem) : occ_one<true, false>(block, smem);
    return savedet ? occ_one<false, true>(block, smem) : occ_one<false, false>(block, smem);
}

}  // namespace umcx_dev
