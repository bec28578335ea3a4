// shape_eval.h - evaluation of the reference's shape constructs at a voxel centre (MCX_userio, fangq/umcx
// src/umcx.cpp:458-473 predicates, L537-604 rasteriser) and of its detector-masking sample test (L605-632), shared
// by the host rasteriser (frontend.cpp, g++ with -ffp-contract=off) and the device rasteriser (raster.cu).
//
// Both sides must give the same label bytes, so every float expression is written with explicitly rounded single
// operations in the reference's evaluation order: on the device __fmul_rn / __fadd_rn / __fsub_rn, which the
// compiler never contracts into a fused multiply-add; on the host plain operators under -ffp-contract=off.
#pragma once

#include <cstdint>

#include "../../include/umcx_gpu.h"

#if defined(__CUDACC__)
#define UMCX_HD __host__ __device__ __forceinline__
#else
#define UMCX_HD inline
#endif

namespace umcx_shape {

#if defined(__CUDA_ARCH__)
UMCX_HD float mul(float a, float b) { return __fmul_rn(a, b); }
UMCX_HD float add(float a, float b) { return __fadd_rn(a, b); }
UMCX_HD float sub(float a, float b) { return __fsub_rn(a, b); }
#else
UMCX_HD float mul(float a, float b) { return a * b; }
UMCX_HD float add(float a, float b) { return a + b; }
UMCX_HD float sub(float a, float b) { return a - b; }
#endif

// Label painted by one op at voxel centre (x, y, z), 0 when outside.  A value the reference would read from a
// missing JSON key (it throws "type must be number, but is null") sets *missing instead; the evaluation order
// and short-circuits are the reference's, so a missing value is reported exactly where the reference reads it.
UMCX_HD int eval_op(const umcx_shape_op& op, float x, float y, float z, bool* missing) {
    const float* f = op.f;
    const bool tag_ok = (op.present & UMCX_SHAPE_HAS_TAG) != 0;
    bool inside = false;
    switch (op.kind) {
        case UMCX_SHAPE_SPHERE: {  // L458-459
            const float dx = sub(x, f[0]), dy = sub(y, f[1]), dz = sub(z, f[2]);
            inside = add(add(mul(dx, dx), mul(dy, dy)), mul(dz, dz)) < mul(f[3], f[3]);
            break;
        }
        case UMCX_SHAPE_BOX: {  // L460: the reference reads "Sip.ze" and compares p.x three times
            if (x < f[0] || y < f[1] || z < f[2]) return 0;
            for (int k = 0; k < 3; k++) {
                if (!(op.present & (UMCX_SHAPE_HAS_SIZE0 << k))) {
                    *missing = true;
                    return 0;
                }
                if (x > add(f[k], f[3 + k])) return 0;
            }
            inside = true;
            break;
        }
        case UMCX_SHAPE_XLAYER:
        case UMCX_SHAPE_YLAYER:
        case UMCX_SHAPE_ZLAYER: {  // L461-463, bounds inclusive
            const float c = op.kind == UMCX_SHAPE_XLAYER ? x : (op.kind == UMCX_SHAPE_YLAYER ? y : z);
            if (!(c >= f[0])) return 0;
            if (!(op.present & UMCX_SHAPE_HAS_HI)) {
                *missing = true;
                return 0;
            }
            inside = c <= f[1];
            break;
        }
        case UMCX_SHAPE_CYLINDER: {  // L464-470: the axial bound compares with the SQUARED axis length
            const float px = sub(x, f[0]), py = sub(y, f[1]), pz = sub(z, f[2]);
            const float d = add(add(mul(f[3], px), mul(f[4], py)), mul(f[5], pz));
            inside = d <= f[6] && d >= 0.f && sub(add(add(mul(px, px), mul(py, py)), mul(pz, pz)), mul(d, d)) <= mul(f[7], f[7]);
            break;
        }
        default:
            return 0;
    }
    if (!inside) return 0;
    if (!tag_ok) {
        *missing = true;
        return 0;
    }
    return op.tag;
}

// Label of voxel (ix, iy, iz) after the Grid fill and every op in order (MCX_volume::mask, L138-140: a shape never
// paints label 0)
UMCX_HD int32_t rasterize_voxel(const umcx_shape_op* ops, int nops, int32_t fill, uint32_t ix, uint32_t iy,
                                uint32_t iz, bool* missing) {
    const float x = add(static_cast<float>(ix), 0.5f), y = add(static_cast<float>(iy), 0.5f),
                z = add(static_cast<float>(iz), 0.5f);
    int32_t label = fill;
    for (int k = 0; k < nops; k++) {
        const int t = eval_op(ops[k], x, y, z, missing);
        if (t) label = t;
    }
    return label;
}

// detector-masking sample test (L613-615): the sample point lies within R + 1 of the detector centre
UMCX_HD bool det_sample_near(float ix, float iy, float iz, float dx, float dy, float dz, float radius) {
    const float ex = sub(ix, dx), ey = sub(iy, dy), ez = sub(iz, dz), r1 = add(radius, 1.f);
    return !(add(add(mul(ex, ex), mul(ey, ey)), mul(ez, ez)) > mul(r1, r1));
}

}  // namespace umcx_shape
