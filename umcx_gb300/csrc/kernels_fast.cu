// kernels_fast.cu - instances of the production (fast-math) propagation kernels, the launch policy and the RNG
// known-answer kernel.
#include <algorithm>

#include "launch.h"

namespace umcx_dev {

template <bool R, bool D>
static void launch_one(const LaunchChoice& lc, const KParams& P, const KBuffers& B, cudaStream_t st) {
    // one-gate volumes (a whole-volume replica or none) take the instances that skip the gate arithmetic
    if (lc.gate1 && lc.rep == kRepWhole) k_forward<false, R, D, kRepWhole, false, true><<<lc.grid, lc.block, lc.smem, st>>>(P, B);
    else if (lc.gate1 && lc.rep == kRepNone) k_forward<false, R, D, kRepNone, false, true><<<lc.grid, lc.block, lc.smem, st>>>(P, B);
    else if (lc.rep == kRepWhole) k_forward<false, R, D, kRepWhole><<<lc.grid, lc.block, lc.smem, st>>>(P, B);
    else if (lc.rep == kRepPrefix) k_forward<false, R, D, kRepPrefix><<<lc.grid, lc.block, lc.smem, st>>>(P, B);
    else if (lc.rep == kRepOff) k_forward<false, R, D, kRepOff><<<lc.grid, lc.block, lc.smem, st>>>(P, B);
    else k_forward<false, R, D><<<lc.grid, lc.block, lc.smem, st>>>(P, B);
}

void launch_forward_fast(const LaunchChoice& lc, const KParams& P, const KBuffers& B, cudaStream_t st) {
    if (lc.aggregate) {
        launch_forward_fast_agg(lc, P, B, st);
        return;
    }
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
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_forward<false, R, D>, block, smem) != cudaSuccess) return 0;
    return n;
}

// allow the forward kernels all the dynamic shared memory a CTA can have (large per-thread partial-path scratch).
// The L1/shared carve-out is left to the driver: preferences from 0 to 40 % shared ran within 1 % of it on the
// benchmark configurations, 60 % was 2 % slower.
template <bool R, bool D>
static cudaError_t allow_big_smem() {
    cudaError_t e = allow_max_dynamic_smem(k_forward<false, R, D>);
    if (e == cudaSuccess) e = allow_max_dynamic_smem(k_forward<false, R, D, kRepPrefix>);
    if (e == cudaSuccess) e = allow_max_dynamic_smem(k_forward<false, R, D, kRepOff>);
    if (e == cudaSuccess) e = allow_max_dynamic_smem(k_forward<false, R, D, kRepNone, false, true>);
    if (e == cudaSuccess) e = allow_max_dynamic_smem(k_forward<false, R, D, kRepWhole, false, true>);
    return e == cudaSuccess ? allow_max_dynamic_smem(k_forward<false, R, D, kRepWhole>) : e;
}
cudaError_t configure_fast_kernels() {
    cudaError_t e = configure_fast_agg_kernels();
    if (e == cudaSuccess) e = allow_big_smem<false, false>();
    if (e == cudaSuccess) e = allow_big_smem<false, true>();
    if (e == cudaSuccess) e = allow_big_smem<true, false>();
    if (e == cudaSuccess) e = allow_big_smem<true, true>();
    return e;
}

int occupancy_fast(bool reflect, bool savedet, int block, size_t smem) {
    if (reflect) return savedet ? occ_one<true, true>(block, smem) : occ_one<true, false>(block, smem);
    return savedet ? occ_one<false, true>(block, smem) : occ_one<false, false>(block, smem);
}

void launch_forward(const LaunchChoice& lc, const KParams& P, const KBuffers& B, cudaStream_t st, bool strict) {
    if (strict) launch_forward_strict(lc, P, B, st);
    else launch_forward_fast(lc, P, B, st);
}

size_t forward_smem(const KParams& P, int block, bool savedet) {
    size_t s = 2 * sizeof(double) * static_cast<size_t>(block);  // per-lane energy tallies
    s += sizeof(Medium) * static_cast<size_t>(P.mediumnum);
    s += sizeof(float) * static_cast<size_t>(block);  // per-lane launch weight
    if (savedet) s += sizeof(float) * static_cast<size_t>(P.ppathlen) * static_cast<size_t>(block);
    s += sizeof(float) * static_cast<size_t>(block);  // aggregation buffer
    return s;
}

int forward_occupancy(bool strict, bool reflect, bool savedet, int block, size_t smem) {
    return strict ? occupancy_strict(reflect, savedet, block, smem) : occupancy_fast(reflect, savedet, block, smem);
}

LaunchChoice choose_launch(int device, int sm_count, const umcx_tuning& t, const umcx_sim* s, const KParams& P) {
    (void)device;
    LaunchChoice lc;
    lc.reflect = s->isreflect != 0;
    lc.savedet = s->issavedet != 0;
    const bool strict = (s->flags & UMCX_SIM_STRICT_MATH) != 0;
    lc.block = t.block_size > 0 ? t.block_size : 1024;  // one CTA of 32 warps per SM: 2-3 % faster than 256
    lc.aggregate = t.aggregation == 2 ? 1 : 0;
    lc.rep = s->issavevol ? kRepNone : kRepOff;  // the caller sets the FP64 volume's replication mode
    lc.gate1 = s->dim[3] == 1;
    lc.smem = forward_smem(P, lc.block, lc.savedet);
    while (lc.smem > kMaxDynamicSmem && lc.block > 32) {  // per-lane partial paths of many media: smaller CTAs
        lc.block /= 2;
        lc.smem = forward_smem(P, lc.block, lc.savedet);
    }
    int occ = forward_occupancy(strict, lc.reflect, lc.savedet, lc.block, lc.smem);
    if (occ < 1) occ = 1;
    const int per_sm = t.blocks_per_sm > 0 ? std::min(t.blocks_per_sm, occ) : occ;
    // a requested grid (the reference's ThreadNum / BlockSize) may exceed one resident wave: the persistent CTAs
    // of later waves start as earlier ones finish and take the photons that are left
    lc.grid = t.grid_size > 0 ? t.grid_size : sm_count * per_sm;
    // never launch more lanes than photons need (small runs): whole warps, at least one CTA
    const unsigned long long lanes = static_cast<unsigned long long>(lc.grid) * lc.block;
    if (P.nphoton < lanes) {
        unsigned long long g = (P.nphoton + lc.block - 1) / lc.block;
        lc.grid = static_cast<int>(std::max<unsigned long long>(1ULL, g));
    }
    return lc;
}

// dst[i] = the FP64 volume rounded once to FP32, its first len elements summed with their reps - 1 copies
// (copy c of element i at n + (c - 1) * len + i)
__global__ void k_fp64_to_fp32(const double* __restrict__ src, float* __restrict__ dst, unsigned long long n,
                               unsigned reps, unsigned long long len) {
    const unsigned long long stride = static_cast<unsigned long long>(gridDim.x) * blockDim.x;
    for (unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += stride) {
        double v = src[i];
        if (i < len)
            for (unsigned r = 1; r < reps; r++) v += src[n + (r - 1) * len + i];
        dst[i] = static_cast<float>(v);
    }
}

void launch_fp64_to_fp32(const double* src, float* dst, unsigned long long n, int sm_count, cudaStream_t stream,
                         Replicas reps) {
    if (n == 0) return;
    const unsigned long long blocks = (n + 255) / 256;
    const int grid = static_cast<int>(blocks < static_cast<unsigned long long>(sm_count) * 8 ? blocks : sm_count * 8ULL);
    k_fp64_to_fp32<<<grid, 256, 0, stream>>>(src, dst, n, reps.copies, reps.copies > 1 ? reps.len : 0ULL);
}

Replicas accumulator_replicas(unsigned long long nvox, unsigned maxgate) {
    const unsigned long long nout = nvox * maxgate;
    unsigned k = 1;
    while (k < kMaxReplicas && 2ULL * k * nout * sizeof(double) <= kReplicaBytes) k *= 2;
    if (k > 1) return Replicas{k, nout};
    // a multi-gate volume: its first gates (the photons' first nanoseconds, still close to the source) in 4 copies
    const unsigned long long gates = kReplicaBytes / sizeof(double) / (3ULL * nvox);
    if (maxgate > 1 && gates >= 1) return Replicas{4u, (gates < maxgate ? gates : maxgate) * nvox};
    return Replicas{1u, 0ULL};
}

__global__ void k_rng_dump(unsigned s0, unsigned s1, unsigned s2, unsigned s3, unsigned long long offset,
                           unsigned nphoton, unsigned ndraw, float* out) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nphoton) return;
    const unsigned long long idx = offset + i;
    const unsigned i32 = static_cast<unsigned>(idx);
    Rng r;
    rng_reseed(r, s0 ^ i32, s1 | i32, s2 ^ i32, s3 | i32);
    float* o = out + static_cast<unsigned long long>(i) * ndraw;
    for (unsigned k = 0; k < ndraw; k++) o[k] = rng_rand01(r);
}

void launch_rng_dump(const uint32_t seeds[4], unsigned long long offset, unsigned nphoton, unsigned ndraw, float* out,
                     cudaStream_t stream) {
    const unsigned block = 128;
    const unsigned grid = (nphoton + block - 1) / block;
    if (grid) k_rng_dump<<<grid, block, 0, stream>>>(seeds[0], seeds[1], seeds[2], seeds[3], offset, nphoton, ndraw, out);
}

}  // namespace umcx_dev
