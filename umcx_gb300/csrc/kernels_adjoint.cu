// kernels_adjoint.cu - instances of the adjoint forward pass, the replay kernel and the reduction of detected-photon
// records into detector readings and their per-label derivatives.
#include "launch.h"

namespace umcx_dev {

size_t adjoint_smem(const KParams& P, int block) {
    const size_t K = static_cast<size_t>(P.mediumnum);
    return (2 * K + 2) * sizeof(double) + K * sizeof(Medium) + static_cast<size_t>(P.ppathlen) * block * sizeof(float) +
           6 * K * block * sizeof(float) + block * sizeof(unsigned long long);  // + photon indices
}

template <bool R>
static cudaError_t allow_adjoint_smem() {
    cudaError_t e = allow_max_dynamic_smem(k_adjoint<R>);
    if (e == cudaSuccess) e = allow_max_dynamic_smem(k_adjoint<R, kRepPrefix>);
    return e == cudaSuccess ? allow_max_dynamic_smem(k_adjoint<R, kRepWhole>) : e;
}

cudaError_t configure_adjoint_kernels() {
    cudaError_t e = allow_adjoint_smem<false>();
    return e == cudaSuccess ? allow_adjoint_smem<true>() : e;
}

int adjoint_occupancy(bool reflect, int block, size_t smem) {
    int n = 0;
    cudaError_t e = reflect ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_adjoint<true>, block, smem)
                            : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_adjoint<false>, block, smem);
    return e == cudaSuccess ? n : 0;
}

template <bool R>
static void launch_adjoint_rep(int grid, int block, size_t smem, int rep, const KParams& P, const KBuffers& B,
                               cudaStream_t st) {
    if (rep == kRepWhole) k_adjoint<R, kRepWhole><<<grid, block, smem, st>>>(P, B);
    else if (rep == kRepPrefix) k_adjoint<R, kRepPrefix><<<grid, block, smem, st>>>(P, B);
    else k_adjoint<R><<<grid, block, smem, st>>>(P, B);
}

void launch_adjoint(int grid, int block, size_t smem, bool reflect, int rep, const KParams& P, const KBuffers& B,
                    cudaStream_t st) {
    if (reflect) launch_adjoint_rep<true>(grid, block, smem, rep, P, B, st);
    else launch_adjoint_rep<false>(grid, block, smem, rep, P, B, st);
}

void launch_replay(int grid, int block, bool reflect, const KParams& P, const KBuffers& B, cudaStream_t st) {
    const size_t smem = sizeof(Medium) * static_cast<size_t>(P.mediumnum);
    if (reflect) k_replay<true><<<grid, block, smem, st>>>(P, B);
    else k_replay<false><<<grid, block, smem, st>>>(P, B);
}

__global__ void k_adjoint_reduce(const KParams P, const DetRecord* __restrict__ rec, const float* __restrict__ ext,
                                 unsigned long long n, const Medium* __restrict__ media, double* __restrict__ read,
                                 double* __restrict__ gmua, double* __restrict__ gmus) {
    const int K = P.mediumnum;
    const unsigned long long stride = static_cast<unsigned long long>(gridDim.x) * blockDim.x;
    for (unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += stride) {
        const DetRecord r = rec[i];
        if (r.det < 1 || r.det > P.detnum) continue;
        const int gate = static_cast<int>(fminf(static_cast<float>(P.maxgate - 1),
                                                floorf((r.time - P.tstart) * P.rtstep)));
        if (gate < 0) continue;
        const unsigned long long cell = static_cast<unsigned long long>(r.det - 1) * P.maxgate + gate;
        const double w = r.weight;
        atomicAdd(read + cell, w);
        const float* e = ext + i * static_cast<unsigned long long>(2 * K);
        for (int k = 0; k < K; k++) {
            const double L = e[k], cnt = e[K + k];
            const double mus = media[k].a.y;
            atomicAdd(gmua + cell * K + k, -w * L);
            atomicAdd(gmus + cell * K + k, w * ((mus > 0.0 ? cnt / mus : 0.0) - L));
        }
    }
}

void launch_adjoint_reduce(const KParams& P, const DetRecord* rec, const float* ext, unsigned long long n,
                           const Medium* media, double* read, double* gmua, double* gmus, int sm_count,
                           cudaStream_t st) {
    if (n == 0) return;
    const unsigned long long blocks = (n + 255) / 256;
    const int grid = static_cast<int>(blocks < 4ULL * sm_count ? blocks : 4ULL * sm_count);
    k_adjoint_reduce<<<grid, 256, 0, st>>>(P, rec, ext, n, media, read, gmua, gmus);
}

}  // namespace umcx_dev
