// kernels_pack.cu - production propagation kernels that read voxel labels from a palette-packed copy of the label
// volume held in shared memory (2 or 4 bits per voxel), and the two small kernels that build that copy.
//
// A voxel crossing needs the label byte of the next voxel.  From global memory that is a dependent load whose
// latency is an L1 hit at best and an L2 round trip when the walk leaves the lines the SM holds; from shared memory
// it is a fixed short load plus a shift and a palette select.  Volumes with few distinct label bytes (a handful of
// tissue labels plus the detector-flagged copies) pack into tens of KB.
#include "launch.h"

namespace umcx_dev {

template <bool R, bool D, int K>
static void launch_one(const LaunchChoice& lc, const KParams& P, const KBuffers& B, cudaStream_t st) {
    k_forward<false, R, D, K><<<lc.grid, lc.block, lc.smem, st>>>(P, B);
}

template <int K>
static void launch_bits(const LaunchChoice& lc, const KParams& P, const KBuffers& B, cudaStream_t st) {
    if (lc.reflect) {
        if (lc.savedet) launch_one<true, true, K>(lc, P, B, st);
        else launch_one<true, false, K>(lc, P, B, st);
    } else {
        if (lc.savedet) launch_one<false, true, K>(lc, P, B, st);
        else launch_one<false, false, K>(lc, P, B, st);
    }
}

void launch_forward_packed(const LaunchChoice& lc, const KParams& P, const KBuffers& B, cudaStream_t st) {
    if (lc.pack == 2) launch_bits<2>(lc, P, B, st);
    else launch_bits<4>(lc, P, B, st);
}

template <bool R, bool D, int K>
static int occ_one(int block, size_t smem) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_forward<false, R, D, K>, block, smem) != cudaSuccess)
        return 0;
    return n;
}

template <int K>
static int occ_bits(bool reflect, bool savedet, int block, size_t smem) {
    if (reflect) return savedet ? occ_one<true, true, K>(block, smem) : occ_one<true, false, K>(block, smem);
    return savedet ? occ_one<false, true, K>(block, smem) : occ_one<false, false, K>(block, smem);
}

int occupancy_packed(bool reflect, bool savedet, int pack, int block, size_t smem) {
    return pack == 2 ? occ_bits<2>(reflect, savedet, block, smem) : occ_bits<4>(reflect, savedet, block, smem);
}

template <bool R, bool D, int K>
static cudaError_t allow_big_smem() {
    return allow_max_dynamic_smem(k_forward<false, R, D, K>);
}

cudaError_t configure_packed_kernels() {
    cudaError_t e = allow_big_smem<false, false, 2>();
    if (e == cudaSuccess) e = allow_big_smem<false, true, 2>();
    if (e == cudaSuccess) e = allow_big_smem<true, false, 2>();
    if (e == cudaSuccess) e = allow_big_smem<true, true, 2>();
    if (e == cudaSuccess) e = allow_big_smem<false, false, 4>();
    if (e == cudaSuccess) e = allow_big_smem<false, true, 4>();
    if (e == cudaSuccess) e = allow_big_smem<true, false, 4>();
    if (e == cudaSuccess) e = allow_big_smem<true, true, 4>();
    return e;
}

// 256-bit set of the label bytes present in the volume.  Labels are spatially coherent, so a lane only touches the
// block's set when its byte differs from the one it recorded last.
__global__ void k_label_presence(const uint8_t* __restrict__ labels, unsigned long long nvox, unsigned* mask) {
    __shared__ unsigned m[8];
    if (threadIdx.x < 8) m[threadIdx.x] = 0u;
    __syncthreads();
    const unsigned long long stride = static_cast<unsigned long long>(gridDim.x) * blockDim.x;
    unsigned last = 256u;
    for (unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < nvox;
         i += stride) {
        const unsigned b = labels[i];
        if (b != last) {
            atomicOr(&m[b >> 5], 1u << (b & 31u));
            last = b;
        }
    }
    __syncthreads();
    if (threadIdx.x < 8 && m[threadIdx.x]) atomicOr(&mask[threadIdx.x], m[threadIdx.x]);
}

// one 32-bit word per lane: 32 / bits consecutive voxels, voxel j of the word in bits [j * bits, (j + 1) * bits)
__global__ void k_label_pack(const uint8_t* __restrict__ labels, unsigned long long nvox, int bits, LabelCodes codes,
                             unsigned* __restrict__ words, unsigned nwords) {
    __shared__ uint8_t code[256];
    for (unsigned k = threadIdx.x; k < 256u; k += blockDim.x) code[k] = codes.c[k];
    __syncthreads();
    const unsigned per = 32u / static_cast<unsigned>(bits);
    for (unsigned w = blockIdx.x * blockDim.x + threadIdx.x; w < nwords; w += gridDim.x * blockDim.x) {
        unsigned v = 0u;
        const unsigned long long first = static_cast<unsigned long long>(w) * per;
        for (unsigned j = 0; j < per; j++) {
            const unsigned long long i = first + j;
            if (i < nvox) v |= static_cast<unsigned>(code[labels[i]]) << (j * static_cast<unsigned>(bits));
        }
        words[w] = v;
    }
}

void launch_label_presence(const uint8_t* labels, unsigned long long nvox, unsigned* mask, int sm_count,
                           cudaStream_t st) {
    if (nvox == 0) return;
    const unsigned long long blocks = (nvox + 255) / 256;
    const int grid = static_cast<int>(blocks < static_cast<unsigned long long>(sm_count) * 4 ? blocks : sm_count * 4ULL);
    k_label_presence<<<grid, 256, 0, st>>>(labels, nvox, mask);
}

void launch_label_pack(const uint8_t* labels, unsigned long long nvox, int bits, const LabelCodes& codes,
                       unsigned* words, unsigned nwords, int sm_count, cudaStream_t st) {
    if (nwords == 0) return;
    const unsigned blocks = (nwords + 255) / 256;
    const int grid = static_cast<int>(blocks < static_cast<unsigned>(sm_count) * 4u ? blocks : sm_count * 4u);
    k_label_pack<<<grid, 256, 0, st>>>(labels, nvox, bits, codes, words, nwords);
}

}  // namespace umcx_dev
