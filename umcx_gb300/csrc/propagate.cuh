// propagate.cuh - device photon engine for sm_103a: the umcx hot path (fangq/umcx src/umcx.cpp:187-440, 752-775)
// as a persistent CUDA kernel.
//
// Per photon the physics is the reference's: the same xorshift128+ stream per photon index (L187-215, L761), the
// same source launch (L225-259), voxel stepping (L315-338), deposition (L359-363), Henyey-Greenstein scattering
// (L364-380), Fresnel reflection/refraction (L381-417) and detection (L429-435), with the reference's quirks kept
// (inverse direction of rotated launches taken from the source direction, no refresh of the inverse direction
// after refraction, reflection snapped with nextafterf towards +-1, ...).
//
// The GPU organisation is new:
//  * persistent grid, one lane = one photon at a time; a lane that finishes takes the next photon index, which it
//    prefetched with an atomic on a global counter when it started the previous one (the atomic's latency is
//    never on the critical path);
//  * the nested photon / scatter / step loops of the reference are flattened into one loop whose iteration is
//    "launch if idle, one voxel step, voxel-crossing handling, scatter if the free path is used up", so lanes of a
//    warp stay busy when their photons are at different stages;
//  * the per-label optical table (with reciprocals and Henyey-Greenstein constants precomputed) sits in shared
//    memory; labels are uint8 loaded through the read-only path;
//  * fluence deposits are issued after the divergent part of the iteration, optionally aggregated per warp with
//    __match_any_sync on the output index; detected photons are appended with a ballot + prefix count per detector;
//  * energy tallies accumulate in FP64 per lane and reach global memory once per warp at exit;
//  * every loop is bounded: a per-photon step cap and a wall-clock deadline (%globaltimer) end the kernel with an
//    error flag instead of hanging.
//
// STRICT = true evaluates every expression like the reference (IEEE division, expf/logf/sinf/cosf/acosf; the
// translation unit is compiled without FMA contraction).  STRICT = false ("fast", the production path) uses the
// hardware approximations __expf/__logf/__sincosf, reciprocal multiplies, and sin(theta) = sqrt(1 - cos^2) instead
// of sincos(acos(cos)): the same distributions, different last bits.
#pragma once

#include <cfloat>
#include <cstdint>

#include "../../include/umcx_gpu.h"

namespace umcx_dev {

constexpr float kOneOverC0 = 3.335640951981520e-12f;  // L29
constexpr float kPi = 3.1415926535897932385f;         // L30
constexpr unsigned kFull = 0xFFFFFFFFu;

enum Kind : int { kForward = 0, kAdjoint = 1, kReplay = 2 };

// per-label optical constants (48 bytes): a = {mua, mus, g, n}; b = {1/mus (0 if mus = 0), 1/mua (0 if mua = 0),
// 1/(2g), n / c0}; c = {1 - g^2, 1 - g, 2g, 1 + g^2}
struct Medium {
    float4 a, b, c;
};

struct KStats {
    double escape;
    double total;
    unsigned long long detected;
    unsigned long long launched;
    unsigned long long steps;
    unsigned long long crossings;
    unsigned long long scatters;
    unsigned long long reflections;
    unsigned long long capped;
    int error;  // 0 ok, 3 deadline reached
    int pad;
};

// extended record of a detected photon (adjoint / replay); per-label path and scatter counts follow in `ext`
struct DetRecord {
    unsigned long long photon;  // photon index (the replay seed)
    int det;                    // detector id (1-based)
    float weight;               // exit weight
    float time;                 // exit time (s)
    float pad;
};

struct KParams {
    int nx, ny, nz, maxgate;
    unsigned dimyz, dimxyz;
    unsigned long long nphoton;
    unsigned long long photon_offset;
    float tstart, tend, rtstep, unitinmm;
    int isreflect, issavevol, issavedet, savedetflag;
    int mediumnum, outputtype, detnum, srctype;
    unsigned maxdetphotons;
    int cols, ppathlen, aggregate;
    unsigned step_cap;
    unsigned seeds[4];
    float4 srcpos, srcdir, srcrdir, srcparam1, srcparam2;
    unsigned long long budget_ns;  // wall-clock budget of the launch (checked against %globaltimer)
    float4 det[UMCX_MAX_DET];
};

struct KBuffers {
    const uint8_t* labels;
    float* fluence;
    double* fluence64;   // optional FP64 accumulation volume (same layout as fluence)
    float* detp;
    const Medium* media;
    KStats* stats;
    unsigned long long* counter;
    // adjoint / replay extras
    DetRecord* detrec;   // [maxdetphotons]
    float* detext;       // [maxdetphotons][2 * mediumnum]: path per label, scatters per label
    double* grad;        // [4][mediumnum] fluence gradients: d/dmua, d/dmus accumulators (see adjoint notes)
    const DetRecord* replay_list;  // replay input
    unsigned long long replay_count;
    float* jacobian;     // replay output [detnum][nx][ny][nz]
};

// ---------------------------------------------------------------- random numbers (MCX_rand, L187-215)
struct Rng {
    unsigned long long t0, t1;
};

__device__ __forceinline__ void rng_reseed(Rng& r, unsigned s0, unsigned s1, unsigned s2, unsigned s3) {
    r.t0 = (static_cast<unsigned long long>(s0) << 32) | s1;
    r.t1 = (static_cast<unsigned long long>(s2) << 32) | s3;
}

__device__ __forceinline__ float rng_rand01(Rng& r) {
    unsigned long long a = r.t0;
    const unsigned long long b = r.t1;
    r.t0 = b;
    a ^= a << 23;
    r.t1 = a ^ b ^ (a >> 18) ^ (b >> 5);
    const unsigned lo = static_cast<unsigned>(r.t1 + b);
    return __uint_as_float(0x3F800000u | (lo >> 9)) - 1.0f;
}

template <bool STRICT>
__device__ __forceinline__ float scat_len(Rng& r) {  // L212-214
    const float u = rng_rand01(r) + FLT_EPSILON;
    if constexpr (STRICT) return -logf(u);
    else return -__logf(u);
}

template <bool STRICT>
__device__ __forceinline__ void sincos_(float a, float* s, float* c) {
    if constexpr (STRICT) {
        *s = sinf(a);
        *c = cosf(a);
    } else {
        __sincosf(a, s, c);
    }
}

template <bool STRICT>
__device__ __forceinline__ float rcp_(float x) {
    if constexpr (STRICT) return 1.f / x;
    else return __fdividef(1.f, x);
}

template <bool STRICT>
__device__ __forceinline__ float rsqrt_(float x) {
    if constexpr (STRICT) return 1.f / sqrtf(x);
    else return rsqrtf(x);
}

__device__ __forceinline__ float sgnf(float v) { return static_cast<float>((v > 0.f) - (v < 0.f)); }

// ---------------------------------------------------------------- photon state (MCX_photon, L218-220)
struct Photon {
    float px, py, pz, pw;  // position, weight
    float vx, vy, vz;      // direction
    float rx, ry, rz;      // inverse direction
    float lx, ly, lz, lw;  // remaining scattering length, time, path since last deposit, weight at last deposit
    int ix, iy, iz, flip;
    int lastvox;
    unsigned media;        // label byte of the current voxel (bit 7 = detector voxel)
    float launchw;
    unsigned nsteps;
    Rng rng;
};

__device__ __forceinline__ int vox_index(const KParams& P, int ix, int iy, int iz) {  // L128-130
    return (ix < 0 || iy < 0 || iz < 0 || ix >= P.nx || iy >= P.ny || iz >= P.nz)
               ? -1
               : static_cast<int>(static_cast<unsigned>(ix) * P.dimyz + static_cast<unsigned>(iy) * static_cast<unsigned>(P.nz) +
                                  static_cast<unsigned>(iz));
}

// rotatevector, L418-428
template <bool STRICT>
__device__ __forceinline__ void rotate(Photon& p, float stheta, float ctheta, float sphi, float cphi) {
    const float vx = p.vx, vy = p.vy, vz = p.vz;
    if (vz > -1.f + FLT_EPSILON && vz < 1.f - FLT_EPSILON) {
        const float tmp0 = 1.f - vz * vz;
        const float tmp1 = STRICT ? stheta / sqrtf(tmp0) : stheta * rsqrtf(tmp0);
        p.vx = tmp1 * (vx * vz * cphi - vy * sphi) + vx * ctheta;
        p.vy = tmp1 * (vy * vz * cphi + vx * sphi) + vy * ctheta;
        p.vz = -tmp1 * tmp0 * cphi + vz * ctheta;
    } else {
        p.vx = stheta * cphi;
        p.vy = stheta * sphi;
        p.vz = (vz > 0.f) ? ctheta : -ctheta;
    }
    const float norm = rsqrt_<STRICT>(p.vx * p.vx + p.vy * p.vy + p.vz * p.vz);
    p.vx *= norm;
    p.vy *= norm;
    p.vz *= norm;
}

// MCX_photon::launch, L225-259; returns the launch weight
template <bool STRICT>
__device__ __forceinline__ float launch(const KParams& P, Photon& p, unsigned long long i) {
    const unsigned i32 = static_cast<unsigned>(i);
    rng_reseed(p.rng, P.seeds[0] ^ i32, P.seeds[1] | i32, P.seeds[2] ^ i32, P.seeds[3] | i32);  // L761
    p.px = P.srcpos.x;
    p.py = P.srcpos.y;
    p.pz = P.srcpos.z;
    p.pw = 1.f;
    p.vx = P.srcdir.x;
    p.vy = P.srcdir.y;
    p.vz = P.srcdir.z;
    const int st = P.srctype;
    if (st == UMCX_SRC_ISOTROPIC || st == UMCX_SRC_CONE) {
        float sphi, cphi, stheta, ctheta;
        sincos_<STRICT>((kPi * 2.f) * rng_rand01(p.rng), &sphi, &cphi);
        if constexpr (STRICT) {
            float th;
            if (st == UMCX_SRC_ISOTROPIC) {
                th = acosf(2.f * rng_rand01(p.rng) - 1.f);
            } else {
                const float c0 = cosf(P.srcparam1.x);
                th = acosf(rng_rand01(p.rng) * (1.0f - c0) + c0);
            }
            stheta = sinf(th);
            ctheta = cosf(th);
        } else {
            if (st == UMCX_SRC_ISOTROPIC) {
                ctheta = 2.f * rng_rand01(p.rng) - 1.f;
            } else {
                const float c0 = cosf(P.srcparam1.x);
                ctheta = rng_rand01(p.rng) * (1.0f - c0) + c0;
            }
            ctheta = fmaxf(-1.f, fminf(1.f, ctheta));
            stheta = sqrtf(fmaxf(0.f, 1.f - ctheta * ctheta));
        }
        rotate<STRICT>(p, stheta, ctheta, sphi, cphi);
    } else if (st == UMCX_SRC_DISK) {
        float sphi, cphi;
        sincos_<STRICT>((kPi * 2.f) * rng_rand01(p.rng), &sphi, &cphi);
        const float r1 = P.srcparam1.x, r2 = P.srcparam1.y;
        const float rad = sqrtf(rng_rand01(p.rng) * fabsf(r1 * r1 - r2 * r2) + r2 * r2);
        if (p.vz > -1.f + FLT_EPSILON && p.vz < 1.f - FLT_EPSILON) {
            const float l = 1.f - p.vz * p.vz;
            const float q = rad / sqrtf(l);
            const float nx = p.px + q * (p.vx * p.vz * cphi - p.vy * sphi);
            const float ny = p.py + q * (p.vy * p.vz * cphi + p.vx * sphi);
            const float nz = p.pz - q * l * cphi;
            p.px = nx;
            p.py = ny;
            p.pz = nz;
        } else {
            p.px += rad * cphi;
            p.py += rad * sphi;
        }
    } else if (st == UMCX_SRC_PLANAR || st == UMCX_SRC_FOURIER) {
        const float a = rng_rand01(p.rng);
        const float b = rng_rand01(p.rng);
        const float4 s1 = P.srcparam1, s2 = P.srcparam2;
        const float nx = p.px + a * s1.x + b * s2.x;
        const float ny = p.py + a * s1.y + b * s2.y;
        const float nz = p.pz + a * s1.z + b * s2.z;
        p.px = nx;
        p.py = ny;
        p.pz = nz;
        if (st == UMCX_SRC_FOURIER) {
            p.pw *= (cosf((floorf(s1.w) * a + floorf(s2.w) * b + s1.w - floorf(s1.w)) * kPi * 2.f) *
                         (1.f - s2.w + floorf(s2.w)) +
                     1.f) *
                    0.5f;
        }
    }
    // inverse direction from the ORIGINAL source direction (L255), also after an isotropic/cone rotation
    p.rx = P.srcrdir.x;
    p.ry = P.srcrdir.y;
    p.rz = P.srcrdir.z;
    p.lx = __int_as_float(0x7fffffff);
    p.ly = 0.f;
    p.lz = 0.f;
    p.lw = p.pw;
    p.ix = static_cast<int>(p.px);
    p.iy = static_cast<int>(p.py);
    p.iz = static_cast<int>(p.pz);
    p.flip = -1;
    p.nsteps = 0;
    return p.pw;
}

// MCX_photon::skip, L339-358: moves a photon launched outside the grid to its entry point; false if it misses
__device__ __forceinline__ bool skip_to_grid(const KParams& P, Photon& p) {
    const float ax = -p.px * p.rx, ay = -p.py * p.ry, az = -p.pz * p.rz;
    const float bx = (static_cast<float>(P.nx) - p.px) * p.rx;
    const float by = (static_cast<float>(P.ny) - p.py) * p.ry;
    const float bz = (static_cast<float>(P.nz) - p.pz) * p.rz;
    const float tmin = fmaxf(fmaxf(fminf(ax, bx), fminf(ay, by)), fminf(az, bz));
    const float tmax = fminf(fminf(fmaxf(ax, bx), fmaxf(ay, by)), fmaxf(az, bz));
    if (tmax < 0.f || tmin > tmax) return false;
    p.px = p.px + tmin * p.vx;
    p.py = p.py + tmin * p.vy;
    p.pz = p.pz + tmin * p.vz;
    p.pw = 1.f;  // the weight is reset to 1 here (L353)
    p.lx = __int_as_float(0x7fffffff);
    p.ly = 0.f;
    p.lz = 0.f;
    p.lw = 1.f;
    p.ix = static_cast<int>(p.px);
    p.iy = static_cast<int>(p.py);
    p.iz = static_cast<int>(p.pz);
    p.flip = -1;
    p.lastvox = vox_index(P, p.ix, p.iy, p.iz);
    return p.lastvox >= 0;
}

// MCX_photon::step, L315-338; returns the new voxel index (lastvox when the step ends inside the voxel).
// *seg returns the distance moved.
template <bool STRICT>
__device__ __forceinline__ int step(const KParams& P, Photon& p, const Medium& m, bool* crossed) {
    const float hx = fabsf((static_cast<float>(p.ix + (p.vx > 0.f)) - p.px) * p.rx);
    const float hy = fabsf((static_cast<float>(p.iy + (p.vy > 0.f)) - p.py) * p.ry);
    const float hz = fabsf((static_cast<float>(p.iz + (p.vz > 0.f)) - p.pz) * p.rz);
    float dist = fminf(fminf(hx, hy), hz);
    p.flip = (dist == hx ? 0 : (dist == hy ? 1 : 2));
    const float mus = m.a.y;
    const float used = fminf(dist * mus, p.lx);
    *crossed = (used != p.lx);
    if constexpr (STRICT) {
        dist = (mus == 0.f) ? dist : (used / mus);
        p.px = p.px + dist * p.vx;
        p.py = p.py + dist * p.vy;
        p.pz = p.pz + dist * p.vz;
        p.pw = p.pw * expf(-m.a.x * dist);
        p.lx -= used;
        p.ly += dist * m.a.w * kOneOverC0;
    } else {
        dist = (mus == 0.f) ? dist : (used * m.b.x);
        p.px = p.px + dist * p.vx;
        p.py = p.py + dist * p.vy;
        p.pz = p.pz + dist * p.vz;
        p.pw = p.pw * __expf(-m.a.x * dist);
        p.lx -= used;
        p.ly += dist * m.b.w;
    }
    p.lz += dist;
    if (*crossed) {
        if (p.flip == 0) p.ix += (p.vx > 0.f ? 1 : -1);
        else if (p.flip == 1) p.iy += (p.vy > 0.f ? 1 : -1);
        else p.iz += (p.vz > 0.f ? 1 : -1);
        return vox_index(P, p.ix, p.iy, p.iz);
    }
    return p.lastvox;
}

// MCX_photon::scatter, L364-380
template <bool STRICT>
__device__ __forceinline__ void scatter(Photon& p, const Medium& m) {
    p.lx = scat_len<STRICT>(p.rng);
    float sphi, cphi, stheta, ctheta;
    sincos_<STRICT>((2.f * kPi) * rng_rand01(p.rng), &sphi, &cphi);
    const float g = m.a.z;
    if constexpr (STRICT) {
        float th;
        if (fabsf(g) > FLT_EPSILON) {
            float t = (1.f - g * g) / (1.f - g + 2.f * g * rng_rand01(p.rng));
            t = (1.f + g * g - t * t) / (2.f * g);
            th = acosf(fmaxf(-1.f, fminf(1.f, t)));
        } else {
            th = acosf(2.f * rng_rand01(p.rng) - 1.f);
        }
        stheta = sinf(th);
        ctheta = cosf(th);
    } else {
        if (fabsf(g) > FLT_EPSILON) {
            const float t = __fdividef(m.c.x, m.c.y + m.c.z * rng_rand01(p.rng));
            ctheta = (m.c.w - t * t) * m.b.z;
        } else {
            ctheta = 2.f * rng_rand01(p.rng) - 1.f;
        }
        ctheta = fmaxf(-1.f, fminf(1.f, ctheta));
        stheta = sqrtf(fmaxf(0.f, 1.f - ctheta * ctheta));
    }
    rotate<STRICT>(p, stheta, ctheta, sphi, cphi);
    p.rx = rcp_<STRICT>(p.vx);
    p.ry = rcp_<STRICT>(p.vy);
    p.rz = rcp_<STRICT>(p.vz);
}

// reflectcoeff + reflect + transmit, L381-417; returns true when the photon is transmitted.  On reflection the
// photon is put back just inside the current voxel and the caller keeps (lastvox, media).
template <bool STRICT>
__device__ __forceinline__ bool reflect(Photon& p, float n1, float n2) {
    const float icos = fabsf((p.flip == 0) ? p.vx : (p.flip == 1 ? p.vy : p.vz));
    const float tmp0 = n1 * n1, tmp1 = n2 * n2;
    float tmp2 = 1.f - tmp0 / tmp1 * (1.f - icos * icos);
    float rtotal = 1.f;
    if (tmp2 > 0.f) {
        float re = tmp0 * icos * icos + tmp1 * tmp2;
        tmp2 = sqrtf(tmp2);
        const float im = 2.f * n1 * n2 * icos * tmp2;
        const float rp = (re - im) / (re + im);
        re = tmp1 * icos * icos + tmp0 * tmp2 * tmp2;
        rtotal = (rp + (re - im) / (re + im)) * 0.5f;
    }
    if (rtotal < 1.f && rng_rand01(p.rng) > rtotal) {  // transmit (L396-404)
        const float k = n1 / n2;
        p.vx *= k;
        p.vy *= k;
        p.vz *= k;
        const float sq = p.vx * p.vx + p.vy * p.vy + p.vz * p.vz;
        if (p.flip == 0) {
            const float t = sq - p.vx * p.vx;
            p.vx = (t < 1.f) ? sqrtf(1.f - t) * sgnf(p.vx) : 0.f;
        } else if (p.flip == 1) {
            const float t = sq - p.vy * p.vy;
            p.vy = (t < 1.f) ? sqrtf(1.f - t) * sgnf(p.vy) : 0.f;
        } else {
            const float t = sq - p.vz * p.vz;
            p.vz = (t < 1.f) ? sqrtf(1.f - t) * sgnf(p.vz) : 0.f;
        }
        const float norm = rsqrt_<STRICT>(p.vx * p.vx + p.vy * p.vy + p.vz * p.vz);
        p.vx *= norm;
        p.vy *= norm;
        p.vz *= norm;
        return true;  // the inverse direction is deliberately left as it was (as in the reference)
    }
    // REFLECT_PHOTON (L31)
    if (p.flip == 0) {
        p.vx = -p.vx;
        p.rx = -p.rx;
        p.px = nextafterf(static_cast<float>(static_cast<int>(p.px + 0.5f)), sgnf(p.vx));
        p.ix = static_cast<int>(p.px);
    } else if (p.flip == 1) {
        p.vy = -p.vy;
        p.ry = -p.ry;
        p.py = nextafterf(static_cast<float>(static_cast<int>(p.py + 0.5f)), sgnf(p.vy));
        p.iy = static_cast<int>(p.py);
    } else {
        p.vz = -p.vz;
        p.rz = -p.rz;
        p.pz = nextafterf(static_cast<float>(static_cast<int>(p.pz + 0.5f)), sgnf(p.vz));
        p.iz = static_cast<int>(p.pz);
    }
    return false;
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

// deposit value of MCX_photon::save (L359-363)
template <bool STRICT>
__device__ __forceinline__ float deposit_value(const KParams& P, const Photon& p, const Medium& m) {
    if (P.outputtype == UMCX_OUT_ENERGY) return p.lw - p.pw;
    if (m.a.x < FLT_EPSILON) return p.lw * p.lz;
    if constexpr (STRICT) return (p.lw - p.pw) / m.a.x;
    else return (p.lw - p.pw) * m.b.y;
}

// one fluence deposit: into the FP64 accumulation volume when the launch has one (converted to the FP32 output
// afterwards), else straight into the FP32 output like the reference (MCX_volume::add, L134-137)
__device__ __forceinline__ void deposit_add(const KBuffers& B, int idx, float v) {
    if (B.fluence64) atomicAdd(B.fluence64 + idx, static_cast<double>(v));
    else atomicAdd(B.fluence + idx, v);
}

__global__ void k_fp64_to_fp32(const double* __restrict__ src, float* __restrict__ dst, unsigned long long n);

// =============================================================================================== the kernel
// Shared memory layout: Medium[mediumnum] | float ppath[ppathlen][blockDim] | float aggbuf[blockDim] (aggregation)
template <bool STRICT, bool REFLECT, bool SAVEDET>
__global__ void __launch_bounds__(1024) k_forward(const KParams P, const KBuffers B) {
    extern __shared__ float4 smem4[];
    Medium* sm = reinterpret_cast<Medium*>(smem4);
    float* ppath = reinterpret_cast<float*>(sm + P.mediumnum);
    float* aggbuf = ppath + (SAVEDET ? P.ppathlen * blockDim.x : 0);
    {
        const float4* src = reinterpret_cast<const float4*>(B.media);
        float4* dst = reinterpret_cast<float4*>(sm);
        for (int k = threadIdx.x; k < 3 * P.mediumnum; k += blockDim.x) dst[k] = src[k];
    }
    __syncthreads();

    const unsigned tid = threadIdx.x;
    const unsigned lane = lane_id();
    const unsigned long long nthreads = static_cast<unsigned long long>(gridDim.x) * blockDim.x;
    const unsigned long long gid = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + tid;
    const unsigned long long N = P.nphoton;

    // the first photon of a lane is its global thread index; later ones come from the counter (offset by nthreads)
    unsigned long long next = gid;
    unsigned long long pending = (gid < N) ? atomicAdd(B.counter, 1ULL) + nthreads : N;

    const unsigned long long t_end = global_ns() + P.budget_ns;
    Photon p;
    p.media = 0;
    p.lastvox = -1;
    bool active = false, done = false;
    double tot = 0.0, esc = 0.0;
    unsigned c_launch = 0, c_steps = 0, c_cross = 0, c_scat = 0, c_refl = 0, c_cap = 0;

    for (unsigned iter = 0;; iter++) {
        // ---- launch a photon on an idle lane (L761-763)
        if (!active && !done) {
            if (next >= N) {
                done = true;
            } else {
                const unsigned long long idx = P.photon_offset + next;
                next = pending;
                pending = (next < N) ? atomicAdd(B.counter, 1ULL) + nthreads : N;
                p.launchw = launch<STRICT>(P, p, idx);
                c_launch++;
                p.lastvox = vox_index(P, p.ix, p.iy, p.iz);
                bool inside = p.lastvox >= 0 || skip_to_grid(P, p);  // L263-267
                if (inside) {
                    p.media = __ldg(B.labels + p.lastvox);
                    p.lx = scat_len<STRICT>(p.rng);
                    if (SAVEDET)
                        for (int k = 0; k < P.ppathlen; k++) ppath[k * blockDim.x + tid] = 0.f;
                    active = true;
                }
            }
        }
        if (__all_sync(kFull, done)) break;
        if ((iter & 1023u) == 0u) {
            const bool late = global_ns() > t_end;
            if (__any_sync(kFull, late)) {
                if (lane == 0) atomicExch(&B.stats->error, UMCX_ERR_TIMEOUT);
                break;
            }
        }

        // ---- one event: a voxel step (+ crossing), then a scatter when the free path is used up
        int dep_idx = -1;
        float dep_val = 0.f;
        bool term = false;
        if (active) {
            if (p.lx > 0.f) {
                const unsigned mid = p.media & UMCX_LABEL_MASK;
                const Medium m = sm[mid];
                bool crossed;
                int newvox = step<STRICT>(P, p, m, &crossed);
                c_steps++;
                if (++p.nsteps > P.step_cap) {
                    term = true;
                    c_cap++;
                } else if (newvox != p.lastvox) {  // L285-310
                    c_cross++;
                    if (SAVEDET && (P.savedetflag & UMCX_DET_PPATH) && mid > 0) ppath[(mid - 1) * blockDim.x + tid] += p.lz;
                    if (P.issavevol) {
                        const int gate = static_cast<int>(fminf(static_cast<float>(P.maxgate - 1),
                                                                static_cast<float>(static_cast<int>(floorf((p.ly - P.tstart) * P.rtstep)))));
                        if (gate >= 0) {
                            dep_idx = p.lastvox + gate * static_cast<int>(P.dimxyz);
                            dep_val = deposit_value<STRICT>(P, p, m);
                        }
                        p.lw = p.pw;
                        p.lz = 0.f;
                    }
                    if (p.ly > P.tend) {
                        term = true;
                    } else {
                        unsigned newmedia = (newvox >= 0) ? __ldg(B.labels + newvox) : 0u;
                        const float n2 = sm[newmedia & UMCX_LABEL_MASK].a.w;
                        if (REFLECT && m.a.w != n2) {
                            c_refl++;
                            if (reflect<STRICT>(p, m.a.w, n2)) {
                                if (newvox < 0 || (newmedia & UMCX_LABEL_MASK) == 0) term = true;
                            } else {
                                newvox = p.lastvox;
                                newmedia = p.media;
                            }
                        } else if (newvox < 0 || ((newmedia & UMCX_LABEL_MASK) == 0 && mid != 0)) {
                            term = true;
                        }
                        if (!term) {
                            p.lastvox = newvox;
                            p.media = newmedia;
                        }
                    }
                }
            }
            if (!term && p.lx <= 0.f) {
                scatter<STRICT>(p, sm[p.media & UMCX_LABEL_MASK]);
                c_scat++;
            }
        }

        // ---- converged part: fluence deposit
        if (P.aggregate) {
            const unsigned hm = __ballot_sync(kFull, dep_idx >= 0);
            if (__popc(hm) > 1) {
                const unsigned grp = __match_any_sync(kFull, dep_idx >= 0 ? static_cast<unsigned>(dep_idx) : 0xFFFFFFFFu);
                aggbuf[tid] = dep_val;
                __syncwarp();
                if (dep_idx >= 0) {
                    const unsigned leader = __ffs(grp) - 1;
                    if (lane == leader) {
                        float s = 0.f;
                        const unsigned base = tid & ~31u;
                        for (unsigned g = grp; g; g &= g - 1) s += aggbuf[base + __ffs(g) - 1];
                        deposit_add(B, dep_idx, s);
                    }
                }
                __syncwarp();
            } else if (dep_idx >= 0) {
                deposit_add(B, dep_idx, dep_val);
            }
        } else if (dep_idx >= 0) {
            deposit_add(B, dep_idx, dep_val);
        }

        // ---- termination: energy tallies (L765-770) and detection (L276-278, L429-435)
        if (SAVEDET) {
            const bool tdet = term && (p.media & UMCX_LABEL_DET) && p.ly <= P.tend;
            if (__any_sync(kFull, tdet)) {
                for (int d = 0; d < P.detnum; d++) {
                    const float4 dp = P.det[d];
                    const bool hit = tdet && ((dp.x - p.px) * (dp.x - p.px) + (dp.y - p.py) * (dp.y - p.py) +
                                                  (dp.z - p.pz) * (dp.z - p.pz) <
                                              dp.w * dp.w);
                    const unsigned hm = __ballot_sync(kFull, hit);
                    if (hm == 0u) continue;
                    const unsigned leader = __ffs(hm) - 1;
                    unsigned long long base = 0;
                    if (lane == leader) base = atomicAdd(&B.stats->detected, static_cast<unsigned long long>(__popc(hm)));
                    base = __shfl_sync(kFull, base, leader);
                    if (hit) {
                        const unsigned long long slot = base + __popc(hm & ((1u << lane) - 1u));
                        if (slot < P.maxdetphotons) {
                            float* rec = B.detp + slot * static_cast<unsigned long long>(P.cols);
                            int k = 0;
                            if (P.savedetflag & UMCX_DET_ID) rec[k++] = static_cast<float>(d + 1);
                            if (P.savedetflag & UMCX_DET_PPATH)
                                for (int q = 0; q < P.ppathlen; q++) rec[k++] = ppath[q * blockDim.x + tid];
                            if (P.savedetflag & UMCX_DET_EXITPOS) {
                                rec[k++] = p.px;
                                rec[k++] = p.py;
                                rec[k++] = p.pz;
                            }
                            if (P.savedetflag & UMCX_DET_EXITDIR) {
                                rec[k++] = p.vx;
                                rec[k++] = p.vy;
                                rec[k++] = p.vz;
                            }
                        }
                    }
                }
            }
        }
        if (term) {
            if ((p.media & UMCX_LABEL_MASK) != 0u) {
                tot += p.launchw;
                esc += p.pw;
            }
            active = false;
        }
    }

    // ---- per-warp reduction of the tallies, one set of atomics per warp
    for (int off = 16; off > 0; off >>= 1) {
        tot += __shfl_down_sync(kFull, tot, off);
        esc += __shfl_down_sync(kFull, esc, off);
        c_launch += __shfl_down_sync(kFull, c_launch, off);
        c_steps += __shfl_down_sync(kFull, c_steps, off);
        c_cross += __shfl_down_sync(kFull, c_cross, off);
        c_scat += __shfl_down_sync(kFull, c_scat, off);
        c_refl += __shfl_down_sync(kFull, c_refl, off);
        c_cap += __shfl_down_sync(kFull, c_cap, off);
    }
    if (lane == 0) {
        atomicAdd(&B.stats->total, tot);
        atomicAdd(&B.stats->escape, esc);
        atomicAdd(&B.stats->launched, static_cast<unsigned long long>(c_launch));
        atomicAdd(&B.stats->steps, static_cast<unsigned long long>(c_steps));
        atomicAdd(&B.stats->crossings, static_cast<unsigned long long>(c_cross));
        atomicAdd(&B.stats->scatters, static_cast<unsigned long long>(c_scat));
        atomicAdd(&B.stats->reflections, static_cast<unsigned long long>(c_refl));
        if (c_cap) atomicAdd(&B.stats->capped, static_cast<unsigned long long>(c_cap));
    }
}

// rand01 known-answer dump (MCX_rand, L187-215)
__global__ void k_rng_dump(unsigned s0, unsigned s1, unsigned s2, unsigned s3, unsigned long long offset,
                           unsigned nphoton, unsigned ndraw, float* out);

}  // namespace umcx_dev
