// next_toward.h - C99 nextafterf for finite arguments, restated from its definition, for host and device code.
#pragma once

#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define UMCX_NT_HD __host__ __device__ __forceinline__
#else
#define UMCX_NT_HD inline
#endif

namespace umcx_dev {

UMCX_NT_HD int32_t float_bits(float x) {
#if defined(__CUDA_ARCH__)
    return __float_as_int(x);
#else
    int32_t i;
    std::memcpy(&i, &x, sizeof(i));
    return i;
#endif
}

UMCX_NT_HD float bits_float(int32_t i) {
#if defined(__CUDA_ARCH__)
    return __int_as_float(i);
#else
    float x;
    std::memcpy(&x, &i, sizeof(x));
    return x;
#endif
}

// y itself when x == y; otherwise the representable float next to x in the direction of y: one unit in the last
// place (adding one to the bit pattern moves away from zero, subtracting one towards it), and from zero the smallest
// subnormal signed like y
UMCX_NT_HD float next_toward(float x, float y) {
    if (x == y) return y;
    if (x == 0.f) return bits_float(static_cast<int32_t>((static_cast<uint32_t>(float_bits(y)) & 0x80000000u) | 1u));
    return bits_float(float_bits(x) + (((x < y) == (x > 0.f)) ? 1 : -1));
}

}  // namespace umcx_dev
