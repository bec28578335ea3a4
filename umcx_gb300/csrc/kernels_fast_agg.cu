// kernels_fast_agg.cu - instances of the production (fast-math) propagation kernel whose fluence deposits are
// aggregated per warp (__match_any_sync on the output index) before the atomics: the autotuner's alternative to plain
// atomics, in a translation unit of its own so that the two sets compile in parallel.
#include "launch.h"

namespace umcx_dev {

template <bool R, bool D>
static void launch_agg(const LaunchChoice& lc, const KParams& P, const KBuffers& B, cudaStream_t st) {
    if (lc.rep == kRepWhole) k_forward<false, R, D, kRepWhole, true><<<lc.grid, lc.block, lc.smem, st>>>(P, B);
    else if (lc.rep == kRepPrefix) k_forward<false, R, D, kRepPrefix, true><<<lc.grid, lc.block, lc.smem, st>>>(P, B);
    else if (lc.rep == kRepOff) k_forward<false, R, D, kRepOff, true><<<lc.grid, lc.block, lc.smem, st>>>(P, B);
    else k_forward<false, R, D, kRepNone, true><<<lc.grid, lc.block, lc.smem, st>>>(P, B);
}

void launch_forward_fast_agg(const LaunchChoice& lc, const KParams& P, const KBuffers& B, cudaStream_t st) {
    if (lc.reflect) {
        if (lc.savedet) launch_agg<true, true>(lc, P, B, st);
        else launch_agg<true, false>(lc, P, B, st);
    } else {
        if (lc.savedet) launch_agg<false, true>(lc, P, B, st);
        else launch_agg<false, false>(lc, P, B, st);
    }
}

template <bool R, bool D>
static cudaError_t allow_big_smem_agg() {
    cudaError_t e = allow_max_dynamic_smem(k_forward<false, R, D, kRepNone, true>);
    if (e == cudaSuccess) e = allow_max_dynamic_smem(k_forward<false, R, D, kRepPrefix, true>);
    if (e == cudaSuccess) e = allow_max_dynamic_smem(k_forward<false, R, D, kRepOff, true>);
    return e == cudaSuccess ? allow_max_dynamic_smem(k_forward<false, R, D, kRepWhole, true>) : e;
}

cudaError_t configure_fast_agg_kernels() {
    cudaError_t e = allow_big_smem_agg<false, false>();
    if (e == cudaSuccess) e = allow_big_smem_agg<false, true>();
    if (e == cudaSuccess) e = allow_big_smem_agg<true, false>();
    if (e == cudaSuccess) e = allow_big_smem_agg<true, true>();
    return e;
}

}  // namespace umcx_dev
