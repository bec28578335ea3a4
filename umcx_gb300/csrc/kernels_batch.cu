// kernels_batch.cu - instances of the batched propagation kernel without detected-photon records, and the batch
// launch helpers.
#include "launch.h"

namespace umcx_dev {

size_t batch_smem(int nsim, int total_media, int total_det, int ppathlen, int block) {
    return sizeof(SimDesc) * static_cast<size_t>(nsim) + sizeof(unsigned long long) * static_cast<size_t>((nsim + 2) & ~1) +
           sizeof(Medium) * static_cast<size_t>(total_media) + sizeof(float4) * static_cast<size_t>(total_det) +
           sizeof(float) * static_cast<size_t>(block) +
           2 * sizeof(double) * static_cast<size_t>(block) +        // per-lane energy tallies
           sizeof(float) * static_cast<size_t>(ppathlen) * block;  // per-lane partial paths
}

cudaError_t configure_batch_kernels() {
    cudaError_t e = allow_max_dynamic_smem(k_batch<false>);
    if (e == cudaSuccess) e = allow_max_dynamic_smem(k_batch<true>);
    if (e == cudaSuccess) e = allow_max_dynamic_smem(k_batch<false, true>);
    if (e == cudaSuccess) e = allow_max_dynamic_smem(k_batch<true, true>);
    if (e == cudaSuccess) e = configure_batch_det_kernels();
    return e;
}

int batch_occupancy(bool reflect, bool savedet, int block, size_t smem) {
    if (savedet) return batch_det_occupancy(reflect, block, smem);
    int n = 0;
    cudaError_t e = reflect ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch<true>, block, smem)
                            : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch<false>, block, smem);
    return e == cudaSuccess ? n : 0;
}

void launch_batch(int grid, int block, size_t smem, bool reflect, const BParams& BP, const KBuffers& B,
                  cudaStream_t st) {
    if (BP.savedet) {  // a chunk with simulations that save detected photons
        launch_batch_det(grid, block, smem, reflect, BP, B, st);
    } else if (BP.aggregate) {  // warp-aggregated deposits (the batch autotuner's alternative to plain atomics)
        if (reflect) k_batch<true, true><<<grid, block, smem, st>>>(BP, B);
        else k_batch<false, true><<<grid, block, smem, st>>>(BP, B);
    } else if (reflect) {
        k_batch<true><<<grid, block, smem, st>>>(BP, B);
    } else {
        k_batch<false><<<grid, block, smem, st>>>(BP, B);
    }
}

}  // namespace umcx_dev
