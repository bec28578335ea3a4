// launch.h - launch configuration and the per-translation-unit kernel launchers.
#pragma once

#include <cuda_runtime.h>

#include "../../include/umcx_gpu.h"
#include "propagate.cuh"

namespace umcx_dev {

// Let a kernel use all the dynamic shared memory a CTA may opt in to, less its static shared memory.
template <class Kernel>
inline cudaError_t allow_max_dynamic_smem(Kernel kernel) {
    int dev = 0, optin = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes fa;
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, kernel);
    if (e != cudaSuccess) return e;
    const int dyn = optin - static_cast<int>(fa.sharedSizeBytes);
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn > 0 ? dyn : 0);
}

struct LaunchChoice {
    int block = 256;
    int grid = 0;
    int aggregate = 0;
    size_t smem = 0;
    bool reflect = false;
    bool savedet = false;
    int rep = kRepNone;  // replication mode of the FP64 output volume (kRepPrefix / kRepWhole: KParams::rep_mask > 0;
                         // kRepOff: no output volume)
    bool gate1 = false;  // the output volume has one time gate
};

// buffer extents (elements) for the device bounds checks of a checked build; nothing in production builds
inline void set_extents(KBuffers& B, unsigned long long labels, unsigned long long out, unsigned long long detp,
                        unsigned long long jacobian) {
#if UMCX_DEVICE_CHECKS
    B.n_labels = labels;
    B.n_out = out;
    B.n_detp = detp;
    B.n_jacobian = jacobian;
#else
    (void)B;
    (void)labels;
    (void)out;
    (void)detp;
    (void)jacobian;
#endif
}

// dynamic shared memory of the forward kernel for a block size
size_t forward_smem(const KParams& P, int block, bool savedet);

// resident CTAs per SM of a forward kernel instance (0 on error)
int forward_occupancy(bool strict, bool reflect, bool savedet, int block, size_t smem);

// grid = SM count x resident CTAs (persistent kernel) unless the tuning names a grid; block size and aggregation
// from the tuning or defaults
LaunchChoice choose_launch(int device, int sm_count, const umcx_tuning& t, const umcx_sim* s, const KParams& P);

void launch_forward(const LaunchChoice& lc, const KParams& P, const KBuffers& B, cudaStream_t stream, bool strict);
void launch_forward_fast(const LaunchChoice& lc, const KParams& P, const KBuffers& B, cudaStream_t stream);
// instances with warp-aggregated fluence deposits (kernels_fast_agg.cu)
void launch_forward_fast_agg(const LaunchChoice& lc, const KParams& P, const KBuffers& B, cudaStream_t stream);
cudaError_t configure_fast_agg_kernels();
void launch_forward_strict(const LaunchChoice& lc, const KParams& P, const KBuffers& B, cudaStream_t stream);
int occupancy_fast(bool reflect, bool savedet, int block, size_t smem);
cudaError_t configure_fast_kernels();
cudaError_t configure_strict_kernels();
int occupancy_strict(bool reflect, bool savedet, int block, size_t smem);

// adjoint forward pass, replay and record reduction (kernels_adjoint.cu)
size_t adjoint_smem(const KParams& P, int block);
cudaError_t configure_adjoint_kernels();
int adjoint_occupancy(bool reflect, int block, size_t smem);
void launch_adjoint(int grid, int block, size_t smem, bool reflect, int rep, const KParams& P, const KBuffers& B,
                    cudaStream_t st);
void launch_replay(int grid, int block, bool reflect, const KParams& P, const KBuffers& B, cudaStream_t st);
void launch_adjoint_reduce(const KParams& P, const DetRecord* rec, const float* ext, unsigned long long n,
                           const Medium* media, double* read, double* gmua, double* gmus, int sm_count,
                           cudaStream_t st);

// batched simulations (kernels_batch.cu; the instances that save detected photons in kernels_batch_det.cu).
// launch_batch runs the record-saving kernel when BP.savedet is set.
size_t batch_smem(int nsim, int total_media, int total_det, int ppathlen, int block);
cudaError_t configure_batch_kernels();
int batch_occupancy(bool reflect, bool savedet, int block, size_t smem);
void launch_batch(int grid, int block, size_t smem, bool reflect, const BParams& BP, const KBuffers& B,
                  cudaStream_t st);
cudaError_t configure_batch_det_kernels();
int batch_det_occupancy(bool reflect, int block, size_t smem);
void launch_batch_det(int grid, int block, size_t smem, bool reflect, const BParams& BP, const KBuffers& B,
                      cudaStream_t st);

// device label builder (raster.cu): one detector's half-voxel sampling lattice, coordinates at coords[off + i]
struct DetLattice {
    float x, y, z, r;  // detector centre and radius
    unsigned xoff, yoff, zoff;
    unsigned nxs, nys, nzs;
};
void launch_raster(const umcx_shape_op* ops, int nops, int32_t fill, const uint32_t dim[3], int32_t* vol,
                   unsigned* missing, int sm_count, cudaStream_t stream);
void launch_mask_det(const int32_t* vol, const uint32_t dim[3], const DetLattice& d, const float* coords,
                     uint8_t* mark, int sm_count, cudaStream_t stream);
void launch_finish_labels(const int32_t* vol, const uint8_t* mark, unsigned long long n, int mediumnum,
                          uint8_t* out, unsigned long long* first_bad, int sm_count, cudaStream_t stream);

// Replicated FP64 accumulation.  With a pencil beam every photon deposits into the same few voxels below the
// source, and their atomics queue at a few L2 slices (see the forward profile of the single-gate configuration).  The
// forward kernel then gives CTA b its own copy (b mod copies) of the first `len` elements of the FP64 volume --
// the whole volume when 8 copies fit in kReplicaBytes of L2, else (several gates) its first gates in 4 copies --
// which splits each hot voxel's atomics over that many addresses; the rounding pass sums the copies.
constexpr unsigned kMaxReplicas = 8;
constexpr unsigned long long kReplicaBytes = 32ULL << 20;
struct Replicas {
    unsigned copies;         // 1: no copies
    unsigned long long len;  // replicated elements at the start of the volume
    int mode(unsigned long long nout) const { return copies < 2 ? kRepNone : (len >= nout ? kRepWhole : kRepPrefix); }
};
Replicas accumulator_replicas(unsigned long long nvox, unsigned maxgate);
void launch_fp64_to_fp32(const double* src, float* dst, unsigned long long n, int sm_count, cudaStream_t stream,
                         Replicas reps = Replicas{1u, 0ULL});

void launch_rng_dump(const uint32_t seeds[4], unsigned long long offset, unsigned nphoton, unsigned ndraw, float* out,
                     cudaStream_t stream);

}  // namespace umcx_dev
