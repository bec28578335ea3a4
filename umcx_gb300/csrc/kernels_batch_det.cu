// kernels_batch_det.cu - instances of the batched propagation kernel that save detected-photon records (a separate
// translation unit so that the batch instances compile in parallel).
#include "launch.h"

namespace umcx_dev {

cudaError_t configure_batch_det_kernels() {
    cudaError_t e = allow_max_dynamic_smem(k_batch<false, false, true>);
    if (e == cudaSuccess) e = allow_max_dynamic_smem(k_batch<true, false, true>);
    if (e == cudaSuccess) e = allow_max_dynamic_smem(k_batch<false, true, true>);
    if (e == cudaSuccess) e = allow_max_dynamic_smem(k_batch<true, true, true>);
    return e;
}

int batch_det_occupancy(bool reflect, int block, size_t smem) {
    int n = 0;
    cudaError_t e = reflect ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch<true, false, true>, block, smem)
                            : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch<false, false, true>, block, smem);
    return e == cudaSuccess ? n : 0;
}

void launch_batch_det(int grid, int block, size_t smem, bool reflect, const BParams& BP, const KBuffers& B,
                      cudaStream_t st) {
    if (BP.aggregate) {
        if (reflect) k_batch<true, true, true><<<grid, block, smem, st>>>(BP, B);
        else k_batch<false, true, true><<<grid, block, smem, st>>>(BP, B);
    } else if (reflect) {
        k_batch<true, false, true><<<grid, block, smem, st>>>(BP, B);
    } else {
        k_batch<false, false, true><<<grid, block, smem, st>>>(BP, B);
    }
}

}  // namespace umcx_dev
