// raster.cu - device label builder: the reference's domain rasteriser (MCX_userio::initdomain, fangq/umcx
// src/umcx.cpp:537-604) and detector masking (L605-632) as three kernels over an int32 working volume.
//
//   k_raster    one lane per voxel: Grid fill, then every shape op in input order (shape_eval.h, the same code the
//               host rasteriser runs), int32 result
//   k_mask_det  one lane per sample point of one detector's half-voxel sampling lattice (the lattice coordinates
//               are generated on the host by the reference's own float accumulation): marks the sampled voxel
//               when it is tissue and touches the boundary or background
//   k_finish    int32 label + mask -> uint8 label | 0x80, with the media-range check of the job set-up
//
// The masking decisions read only `label & 0x7FFFFFFF`, which marking never changes, so the lanes' order does not
// matter and a byte store of 1 per hit is enough.
#include "launch.h"
#include "shape_eval.h"

namespace umcx_dev {

__global__ void k_raster(const umcx_shape_op* __restrict__ ops, int nops, int32_t fill, uint32_t nx, uint32_t ny,
                         uint32_t nz, int32_t* __restrict__ vol, unsigned* __restrict__ missing) {
    const unsigned long long n = 1ULL * nx * ny * nz;
    const unsigned long long stride = static_cast<unsigned long long>(gridDim.x) * blockDim.x;
    bool miss = false;
    for (unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += stride) {
        const uint32_t iz = static_cast<uint32_t>(i % nz);
        const unsigned long long r = i / nz;
        const uint32_t iy = static_cast<uint32_t>(r % ny);
        const uint32_t ix = static_cast<uint32_t>(r / ny);
        vol[i] = umcx_shape::rasterize_voxel(ops, nops, fill, ix, iy, iz, &miss);
    }
    if (miss) atomicOr(missing, 1u);
}

// LabelVolume::index / MCX_volume::index (L128-130): 16-bit coordinates against 16-bit sizes, -1 outside
__device__ __forceinline__ long long index16(int ix, int iy, int iz, uint32_t nx, uint32_t ny, uint32_t nz) {
    const int16_t sx = static_cast<int16_t>(ix), sy = static_cast<int16_t>(iy), sz = static_cast<int16_t>(iz);
    if (sx < 0 || sy < 0 || sz < 0 || sx >= static_cast<int16_t>(nx) || sy >= static_cast<int16_t>(ny) ||
        sz >= static_cast<int16_t>(nz))
        return -1;
    return static_cast<long long>(sx) * ny * nz + static_cast<long long>(sy) * nz + sz;
}

__global__ void k_mask_det(const int32_t* __restrict__ vol, uint32_t nx, uint32_t ny, uint32_t nz, DetLattice d,
                           const float* __restrict__ coords, uint8_t* __restrict__ mark) {
    // the 26 neighbour offsets in the reference's order (L606)
    constexpr int8_t nb[26][3] = {{-1, -1, -1}, {0, -1, -1}, {1, -1, -1}, {-1, 0, -1}, {0, 0, -1}, {1, 0, -1},
                                  {-1, 1, -1},  {0, 1, -1},  {1, 1, -1},  {-1, -1, 0}, {0, -1, 0}, {1, -1, 0},
                                  {-1, 0, 0},   {1, 0, 0},   {-1, 1, 0},  {0, 1, 0},   {1, 1, 0},  {-1, -1, 1},
                                  {0, -1, 1},   {1, -1, 1},  {-1, 0, 1},  {0, 0, 1},   {1, 0, 1},  {-1, 1, 1},
                                  {0, 1, 1},    {1, 1, 1}};
    const unsigned long long total = 1ULL * nx * ny * nz;
    const unsigned long long n = 1ULL * d.nxs * d.nys * d.nzs;
    const unsigned long long stride = static_cast<unsigned long long>(gridDim.x) * blockDim.x;
    for (unsigned long long t = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x; t < n;
         t += stride) {
        const float fx = coords[d.xoff + t % d.nxs];
        const float fy = coords[d.yoff + (t / d.nxs) % d.nys];
        const float fz = coords[d.zoff + t / (1ULL * d.nxs * d.nys)];
        // (short) conversion of the sample coordinates (L612), through int like the host compilers
        const int16_t sx = static_cast<int16_t>(static_cast<int>(fx)), sy = static_cast<int16_t>(static_cast<int>(fy)),
                      sz = static_cast<int16_t>(static_cast<int>(fz));
        const long long idx = index16(sx, sy, sz, nx, ny, nz);
        if (idx < 0 || !umcx_shape::det_sample_near(fx, fy, fz, d.x, d.y, d.z, d.r) || (vol[idx] & 0x7FFFFFFF) == 0)
            continue;
        if (static_cast<int>(sx) * sy * sz == 0 || sx == static_cast<int16_t>(nx) || sy == static_cast<int16_t>(ny) ||
            sz == static_cast<int16_t>(nz)) {
            mark[idx] = 1;
            continue;
        }
        for (int k = 0; k < 26; k++) {
            // the reference offsets by index(dx, dy, dz), which is -1 whenever a component is negative (L620);
            // neighbours beyond the array count as background
            const long long j = idx + index16(nb[k][0], nb[k][1], nb[k][2], nx, ny, nz);
            const int32_t lab = (j >= 0 && static_cast<unsigned long long>(j) < total) ? vol[j] : 0;
            if ((lab & 0x7FFFFFFF) == 0) {
                mark[idx] = 1;
                break;
            }
        }
    }
}

__global__ void k_finish(const int32_t* __restrict__ vol, const uint8_t* __restrict__ mark, unsigned long long n,
                         int mediumnum, uint8_t* __restrict__ out, unsigned long long* __restrict__ first_bad) {
    const unsigned long long stride = static_cast<unsigned long long>(gridDim.x) * blockDim.x;
    for (unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += stride) {
        const int32_t v = vol[i];
        const int32_t med = v & 0x7FFFFFFF;
        if (med >= mediumnum || med > static_cast<int32_t>(UMCX_LABEL_MASK)) atomicMin(first_bad, i);
        const bool det = mark[i] != 0 || (v & static_cast<int32_t>(0x80000000u)) != 0;
        out[i] = static_cast<uint8_t>((med & 0xFF) | (det ? UMCX_LABEL_DET : 0u));
    }
}

static int grid_for(unsigned long long n, int sm_count) {
    const unsigned long long blocks = (n + 255) / 256;
    const unsigned long long cap = static_cast<unsigned long long>(sm_count) * 8ULL;
    return static_cast<int>(blocks < 1 ? 1 : (blocks < cap ? blocks : cap));
}

void launch_raster(const umcx_shape_op* ops, int nops, int32_t fill, const uint32_t dim[3], int32_t* vol,
                   unsigned* missing, int sm_count, cudaStream_t st) {
    const unsigned long long n = 1ULL * dim[0] * dim[1] * dim[2];
    k_raster<<<grid_for(n, sm_count), 256, 0, st>>>(ops, nops, fill, dim[0], dim[1], dim[2], vol, missing);
}

void launch_mask_det(const int32_t* vol, const uint32_t dim[3], const DetLattice& d, const float* coords,
                     uint8_t* mark, int sm_count, cudaStream_t st) {
    const unsigned long long n = 1ULL * d.nxs * d.nys * d.nzs;
    if (n == 0) return;
    k_mask_det<<<grid_for(n, sm_count), 256, 0, st>>>(vol, dim[0], dim[1], dim[2], d, coords, mark);
}

void launch_finish_labels(const int32_t* vol, const uint8_t* mark, unsigned long long n, int mediumnum,
                          uint8_t* out, unsigned long long* first_bad, int sm_count, cudaStream_t st) {
    k_finish<<<grid_for(n, sm_count), 256, 0, st>>>(vol, mark, n, mediumnum, out, first_bad);
}

}  // namespace umcx_dev
