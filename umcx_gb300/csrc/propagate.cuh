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
//    __match_any_sync on the output index; detected photons are appended, by the lanes that end a photon, with a
//    ballot + prefix count per detector and one atomic per warp;
//  * energy tallies accumulate in FP64 per lane and reach global memory once per warp at exit;
//  * every loop is bounded: a per-photon step cap and a wall-clock deadline (%globaltimer) end the kernel with an
//    error flag instead of hanging.
//
// STRICT = true evaluates every expression like the reference (IEEE division, expf/logf/sinf/cosf/acosf; the
// translation unit is compiled without FMA contraction).  STRICT = false ("fast", the production path) uses the
// hardware approximations __expf/__logf/__sincosf, reciprocal multiplies, and sin(theta) = sqrt(1 - cos^2) instead
// of sincos(acos(cos)), and its translation units are compiled with --use_fast_math (single-precision denormals
// flushed to zero): the same distributions, different last bits.
#pragma once

#include <cfloat>
#include <cstdint>

#include "../../include/umcx_gpu.h"
#include "next_toward.h"

namespace umcx_dev {

constexpr float kOneOverC0 = 3.335640951981520e-12f;  // L29
constexpr float kPi = 3.1415926535897932385f;         // L30
constexpr unsigned kFull = 0xFFFFFFFFu;
constexpr unsigned kZeroStepLimit = 255;  // consecutive zero-length steps before a photon is stopped
constexpr unsigned kDefaultStepCap = 1u << 24;  // steps of one photon before it is stopped

enum Kind : int { kForward = 0, kAdjoint = 1, kReplay = 2 };

// per-label optical constants (48 bytes): a = {mua, mus, g, n}; b = {1/mus (0 if mus = 0), deposit factor,
// 1/(2g), n / c0}; c = {1 - g^2, 1 - g, 2g, 1 + g^2}
struct Medium {
    float4 a, b, c;
};

// Factor of MCX_photon::save's deposit (L359-363) for an output type: the weight loss itself for energy output,
// divided by mua for fluence and fluence rate, and -1 (deposit weight x path length instead) when mua < FLT_EPSILON
__host__ __device__ inline float deposit_factor(float mua, int outputtype) {
    if (outputtype == UMCX_OUT_ENERGY) return 1.f;
    return mua < FLT_EPSILON ? -1.f : 1.f / mua;
}

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
    int error;  // 0 ok, 3 deadline reached, kCheckError + site: a failed device bounds check (checked builds)
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
    unsigned seeds[4];
    float4 srcpos, srcdir, srcrdir, srcparam1, srcparam2;
    unsigned long long budget_ns;  // wall-clock budget of the launch (checked against %globaltimer)
    unsigned rep_mask;             // forward kernel: CTA b deposits into copy c = b & rep_mask of the first rep_len
    unsigned rep_len;              // elements of the FP64 volume (copy 0 is the volume itself; see accumulator_replicas)
    float gate_off;                // -tstart * rtstep: the fast kernels' time gate is t * rtstep + gate_off
    float4 det[UMCX_MAX_DET];
};

// ---------------------------------------------------------------- device bounds checks (checked build variant)
// Built with UMCX_DEVICE_CHECKS=1 (e.g. UMCX_NVCC_DEFS="UMCX_DEVICE_CHECKS=1"), the kernels test every indexed
// access of a device buffer -- label reads (and the medium each label names), output deposits, detected-photon rows
// and Jacobian adds -- against the buffer's extent first (partial-path slots are bounded by ppathlen in every
// build; kSitePath keeps its number for the host's site names).  An access outside it is skipped and
// recorded in KStats::error as kCheckError + site (the first miss wins); the host turns it into an error naming the
// site.  Production builds compile none of it.
#ifndef UMCX_DEVICE_CHECKS
#define UMCX_DEVICE_CHECKS 0
#endif
enum CheckSite { kSiteLabel = 0, kSiteMedium = 1, kSiteOutput = 2, kSitePath = 3, kSiteDetRow = 4, kSiteJacobian = 5 };
constexpr int kCheckError = 16;

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
#if UMCX_DEVICE_CHECKS
    // element counts of the buffers above for the device bounds checks.  Checked builds only: extra kernel-parameter
    // bytes alone changed the register allocation of the production adjoint kernel (spills)
    unsigned long long n_labels, n_out, n_detp, n_jacobian;
#endif
};
// extent of a KBuffers buffer for index_ok (0 in production builds, where index_ok ignores it)
#if UMCX_DEVICE_CHECKS
#define UMCX_EXTENT(B, field) ((B).field)
#else
#define UMCX_EXTENT(B, field) 0ULL
#endif


// true when i < n; in a checked build a miss is recorded in *err and the caller skips the access
__device__ __forceinline__ bool index_ok(int* err, unsigned long long i, unsigned long long n, int site) {
    if constexpr (UMCX_DEVICE_CHECKS != 0) {
        if (i >= n) {
            atomicCAS(err, 0, kCheckError + site);
            return false;
        }
    }
    (void)err;
    (void)i;
    (void)n;
    (void)site;
    return true;
}

// ---------------------------------------------------------------- random numbers (MCX_rand, L187-215)
struct Rng {
    unsigned long long t0, t1;
};

__device__ __forceinline__ void rng_reseed(Rng& r, unsigned s0, unsigned s1, unsigned s2, unsigned s3) {
    r.t0 = (static_cast<unsigned long long>(s0) << 32) | s1;
    r.t1 = (static_cast<unsigned long long>(s2) << 32) | s3;
}

// one xorshift128+ draw as the float 1 + (23 random bits) / 2^23 in [1, 2); rng_rand01 subtracts the 1 (exactly)
__device__ __forceinline__ float rng_rand12(Rng& r) {
    unsigned long long a = r.t0;
    const unsigned long long b = r.t1;
    r.t0 = b;
    a ^= a << 23;
    r.t1 = a ^ b ^ (a >> 18) ^ (b >> 5);
    const unsigned lo = static_cast<unsigned>(r.t1 + b);
    return __uint_as_float(0x3F800000u | (lo >> 9));
}

__device__ __forceinline__ float rng_rand01(Rng& r) { return rng_rand12(r) - 1.0f; }

template <bool STRICT>
__device__ __forceinline__ float scat_len(Rng& r) {  // L212-214
    if constexpr (STRICT) {
        return -logf(rng_rand01(r) + FLT_EPSILON);
    } else {
        // (f - 1) + 2^-23 and f + (2^-23 - 1) are both exact for f = 1 + k 2^-23 (k < 2^23): one addition instead of two
        return -__logf(rng_rand12(r) + (FLT_EPSILON - 1.0f));
    }
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

// The engine functions below are templates over the parameter view PV: KParams (one simulation, kernel
// parameter) or SimDesc (one simulation of a batch, shared memory); both expose the same member names.
template <class PV>
__device__ __forceinline__ int vox_index(const PV& P, int ix, int iy, int iz) {  // L128-130
    // one unsigned compare per axis covers both bounds
    return (static_cast<unsigned>(ix) < static_cast<unsigned>(P.nx) && static_cast<unsigned>(iy) < static_cast<unsigned>(P.ny) &&
            static_cast<unsigned>(iz) < static_cast<unsigned>(P.nz))
               ? static_cast<int>(static_cast<unsigned>(ix) * P.dimyz + static_cast<unsigned>(iy) * static_cast<unsigned>(P.nz) +
                                  static_cast<unsigned>(iz))
               : -1;
}

// rotatevector, L418-428
template <bool STRICT>
__device__ __forceinline__ void rotate(Photon& p, float stheta, float ctheta, float sphi, float cphi) {
    const float vx = p.vx, vy = p.vy, vz = p.vz;
    if (vz > -1.f + FLT_EPSILON && vz < 1.f - FLT_EPSILON) {
        const float tmp0 = 1.f - vz * vz;
        const float tmp1 = STRICT ? stheta / sqrtf(tmp0) : stheta * rsqrtf(tmp0);
        if constexpr (STRICT) {
            p.vx = tmp1 * (vx * vz * cphi - vy * sphi) + vx * ctheta;
            p.vy = tmp1 * (vy * vz * cphi + vx * sphi) + vy * ctheta;
        } else {  // x and y as packed FP32x2 operations
            const float2 vxy = make_float2(vx, vy);
            const float vzc = vz * cphi;
            const float2 a = __ffma2_rn(vxy, make_float2(vzc, vzc), __fmul2_rn(make_float2(-vy, vx), make_float2(sphi, sphi)));
            const float2 r = __ffma2_rn(make_float2(tmp1, tmp1), a, __fmul2_rn(vxy, make_float2(ctheta, ctheta)));
            p.vx = r.x;
            p.vy = r.y;
        }
        p.vz = -tmp1 * tmp0 * cphi + vz * ctheta;
    } else {
        p.vx = stheta * cphi;
        p.vy = stheta * sphi;
        p.vz = (vz > 0.f) ? ctheta : -ctheta;
    }
    if constexpr (STRICT) {
        const float norm = rsqrt_<STRICT>(p.vx * p.vx + p.vy * p.vy + p.vz * p.vz);
        p.vx *= norm;
        p.vy *= norm;
        p.vz *= norm;
    } else {
        const float2 sq = __fmul2_rn(make_float2(p.vx, p.vy), make_float2(p.vx, p.vy));
        const float norm = rsqrtf(sq.x + sq.y + p.vz * p.vz);
        const float2 vxy = __fmul2_rn(make_float2(p.vx, p.vy), make_float2(norm, norm));
        p.vx = vxy.x;
        p.vy = vxy.y;
        p.vz *= norm;
    }
}

// MCX_photon::launch, L225-259; returns the launch weight
template <bool STRICT, class PV>
__device__ __forceinline__ float launch(const PV& P, Photon& p, unsigned long long i) {
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
template <class PV>
__device__ __forceinline__ bool skip_to_grid(const PV& P, Photon& p) {
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
template <bool STRICT, class PV>
__device__ __forceinline__ int step(const PV& P, Photon& p, const Medium& m, bool* crossed, float* moved) {
    const int bx = p.vx > 0.f, by = p.vy > 0.f, bz = p.vz > 0.f;
    // x and y as packed FP32x2 operations (each component rounded like the scalar operation)
    const float2 hxy = __fmul2_rn(__fadd2_rn(make_float2(static_cast<float>(p.ix + bx), static_cast<float>(p.iy + by)),
                                             make_float2(-p.px, -p.py)),
                                  make_float2(p.rx, p.ry));
    const float hx = fabsf(hxy.x), hy = fabsf(hxy.y);
    const float hz = fabsf((static_cast<float>(p.iz + bz) - p.pz) * p.rz);
    float dist = fminf(fminf(hx, hy), hz);
    p.flip = (dist == hx ? 0 : (dist == hy ? 1 : 2));
    const float mus = m.a.y;
    const float used = fminf(dist * mus, p.lx);
    *crossed = (used != p.lx);
    if constexpr (STRICT) {
        dist = (mus == 0.f) ? dist : (used / mus);
        const float2 pxy = __fadd2_rn(make_float2(p.px, p.py), __fmul2_rn(make_float2(dist, dist), make_float2(p.vx, p.vy)));
        p.px = pxy.x;
        p.py = pxy.y;
        p.pz = p.pz + dist * p.vz;
        p.pw = p.pw * expf(-m.a.x * dist);
        p.lx -= used;
        p.ly += dist * m.a.w * kOneOverC0;
    } else {
        // a crossing step moves the wall distance itself (the reference's used / mus is that distance rounded
        // twice; with mus = 0 it is the only choice); otherwise the free path used / mus.  A free path of 0 (a draw
        // of -log(1)) therefore moves nothing, which lets photon_step run the step without testing lx > 0 first.
        dist = *crossed ? dist : used * m.b.x;
        const float2 pxy = __ffma2_rn(make_float2(dist, dist), make_float2(p.vx, p.vy), make_float2(p.px, p.py));
        p.px = pxy.x;
        p.py = pxy.y;
        p.pz = p.pz + dist * p.vz;
        p.pw = p.pw * __expf(-m.a.x * dist);
        p.lx -= used;
        p.ly += dist * m.b.w;
    }
    p.lz += dist;
    *moved = dist;
    // branch-free voxel update: +-1 on the crossed axis only
    const int f = p.flip;
    const int c = *crossed;
    p.ix += (c & (f == 0)) * (2 * bx - 1);
    p.iy += (c & (f == 1)) * (2 * by - 1);
    p.iz += (c & (f == 2)) * (2 * bz - 1);
    return c ? vox_index(P, p.ix, p.iy, p.iz) : p.lastvox;
}

// MCX_photon::scatter, L364-380
template <bool STRICT>
__device__ __forceinline__ void scatter(Photon& p, const Medium& m) {
    p.lx = scat_len<STRICT>(p.rng);
    float sphi, cphi, stheta, ctheta;
    if constexpr (STRICT) {
        sincos_<STRICT>((2.f * kPi) * rng_rand01(p.rng), &sphi, &cphi);
    } else {
        // 2 pi (f - 1) with f - 1 exact, as one fused multiply-add with the same single rounding
        sincos_<STRICT>(fmaf(rng_rand12(p.rng), 2.f * kPi, -2.f * kPi), &sphi, &cphi);
    }
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
        // both cases draw one number: select instead of branching (lanes in different media do not diverge)
        const float r = rng_rand01(p.rng);
        const float t = __fdividef(m.c.x, m.c.y + m.c.z * r);
        ctheta = fabsf(g) > FLT_EPSILON ? (m.c.w - t * t) * m.b.z : 2.f * r - 1.f;
        ctheta = fmaxf(-1.f, fminf(1.f, ctheta));
        const float s2 = fmaxf(0.f, 1.f - ctheta * ctheta);
        stheta = sqrtf(s2);
    }
    rotate<STRICT>(p, stheta, ctheta, sphi, cphi);
    p.rx = rcp_<STRICT>(p.vx);
    p.ry = rcp_<STRICT>(p.vy);
    p.rz = rcp_<STRICT>(p.vz);
}

template <bool STRICT>
__device__ __forceinline__ float div_(float a, float b) {
    if constexpr (STRICT) return a / b;
    else return __fdividef(a, b);
}

// square root of a positive argument
template <bool STRICT>
__device__ __forceinline__ float sqrt_pos_(float x) {
    if constexpr (STRICT) return sqrtf(x);
    else return x * rsqrtf(x);
}

template <bool STRICT>
__device__ __forceinline__ float nextafter_(float x, float y) {
    if constexpr (STRICT) return nextafterf(x, y);
    else return next_toward(x, y);
}

// reflectcoeff + reflect + transmit, L381-417; returns true when the photon is transmitted.  On reflection the
// photon is put back just inside the current voxel and the caller keeps (lastvox, media).  The crossed axis (flip)
// is selected arithmetically rather than by branches: this block runs in about a third of the warp iterations
// (2 % of crossings reflect, but any lane of the warp brings the whole warp through it).
template <bool STRICT>
__device__ __forceinline__ bool reflect(Photon& p, float n1, float n2) {
    const int f = p.flip;
    const float icos = fabsf((f == 0) ? p.vx : (f == 1 ? p.vy : p.vz));
    const float tmp0 = n1 * n1, tmp1 = n2 * n2;
    float tmp2 = 1.f - div_<STRICT>(tmp0, tmp1) * (1.f - icos * icos);
    float rtotal = 1.f;
    if (tmp2 > 0.f) {
        float re = tmp0 * icos * icos + tmp1 * tmp2;
        tmp2 = sqrt_pos_<STRICT>(tmp2);
        const float im = 2.f * n1 * n2 * icos * tmp2;
        const float rp = div_<STRICT>(re - im, re + im);
        re = tmp1 * icos * icos + tmp0 * tmp2 * tmp2;
        rtotal = (rp + div_<STRICT>(re - im, re + im)) * 0.5f;
    }
    if (rtotal < 1.f && rng_rand01(p.rng) > rtotal) {  // transmit (L396-404)
        const float k = div_<STRICT>(n1, n2);
        p.vx *= k;
        p.vy *= k;
        p.vz *= k;
        const float sq = p.vx * p.vx + p.vy * p.vy + p.vz * p.vz;
        const float vc = (f == 0) ? p.vx : (f == 1 ? p.vy : p.vz);
        const float t = sq - vc * vc;
        const float nv = (t < 1.f) ? sqrt_pos_<STRICT>(1.f - t) * sgnf(vc) : 0.f;
        p.vx = (f == 0) ? nv : p.vx;
        p.vy = (f == 1) ? nv : p.vy;
        p.vz = (f == 2) ? nv : p.vz;
        const float norm = rsqrt_<STRICT>(p.vx * p.vx + p.vy * p.vy + p.vz * p.vz);
        p.vx *= norm;
        p.vy *= norm;
        p.vz *= norm;
        return true;  // the inverse direction is deliberately left as it was (as in the reference)
    }
    // REFLECT_PHOTON (L31): the crossed axis' direction and inverse direction change sign, the position snaps to the
    // nearest voxel face and moves one float towards the new direction
    const float vc = -((f == 0) ? p.vx : (f == 1 ? p.vy : p.vz));
    const float pc = (f == 0) ? p.px : (f == 1 ? p.py : p.pz);
    const float np = nextafter_<STRICT>(static_cast<float>(static_cast<int>(pc + 0.5f)), sgnf(vc));
    const int ni = static_cast<int>(np);
    p.vx = (f == 0) ? vc : p.vx;
    p.vy = (f == 1) ? vc : p.vy;
    p.vz = (f == 2) ? vc : p.vz;
    p.rx = (f == 0) ? -p.rx : p.rx;
    p.ry = (f == 1) ? -p.ry : p.ry;
    p.rz = (f == 2) ? -p.rz : p.rz;
    p.px = (f == 0) ? np : p.px;
    p.py = (f == 1) ? np : p.py;
    p.pz = (f == 2) ? np : p.pz;
    p.ix = (f == 0) ? ni : p.ix;
    p.iy = (f == 1) ? ni : p.iy;
    p.iz = (f == 2) ? ni : p.iz;
    return false;
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

// deposit value of MCX_photon::save (L359-363).  The fast path reads the output type and the mua < FLT_EPSILON case
// from the medium's deposit factor (Medium.b.y, see deposit_factor); the strict path evaluates them like the reference.
template <bool STRICT, class PV>
__device__ __forceinline__ float deposit_value(const PV& P, const Photon& p, const Medium& m) {
    if constexpr (STRICT) {
        if (P.outputtype == UMCX_OUT_ENERGY) return p.lw - p.pw;
        if (m.a.x < FLT_EPSILON) return p.lw * p.lz;
        return (p.lw - p.pw) / m.a.x;
    } else {
        const float f = m.b.y;
        return f < 0.f ? p.lw * p.lz : (p.lw - p.pw) * f;
    }
}

// The CTA's copy of the replicated part of an FP64 volume: deposits below `len` go `base` elements further
// (len = 0: no copy, every deposit goes to the volume itself).  Kernels are instantiated per replication mode:
// kRepNone, kRepPrefix (the first gates are replicated: one compare per deposit) or kRepWhole (every element is).
// kRepOff marks a launch that saves no output volume (issavevol 0), so that the forward kernels know at compile time
// whether a crossing deposits.
enum { kRepNone = 0, kRepPrefix = 1, kRepWhole = 2, kRepOff = 3 };
struct Replica {
    unsigned len;
    unsigned base;  // below 2^32: the volume is below 2^31 elements and its copies below 4 Mi elements
};
template <int REP>
__device__ __forceinline__ Replica cta_replica(const KParams& P) {
    Replica r{0u, 0u};
    if (REP == kRepPrefix || REP == kRepWhole) {  // copy c >= 1 of the CTA lies after the volume and copies 1 .. c-1
        const unsigned c = blockIdx.x & P.rep_mask;
        // copy 0 is the volume itself (base 0), so every CTA can compare with the kernel parameter: the length is
        // then read from the constant bank and the loop keeps one register (base) for the replica (-1.1 % at
        // configuration 2)
        r.len = P.rep_len;
        r.base = c ? P.dimxyz * static_cast<unsigned>(P.maxgate) + (c - 1u) * P.rep_len : 0u;
    }
    return r;
}

// one fluence deposit: into the FP64 accumulation volume when the launch has one (converted to the FP32 output
// afterwards), else straight into the FP32 output like the reference (MCX_volume::add, L134-137)
template <int REP = kRepNone>
__device__ __forceinline__ void deposit_add(const KBuffers& B, int idx, float v, Replica rep = Replica{0u, 0u}) {
    if constexpr (REP == kRepOff) return;  // no output volume
    if (!index_ok(&B.stats->error, static_cast<unsigned long long>(static_cast<long long>(idx)), UMCX_EXTENT(B, n_out),
                  kSiteOutput))
        return;
    if (REP != kRepNone || B.fluence64) {  // a replicated volume is always the FP64 accumulator
        if (REP == kRepNone) {
            atomicAdd(B.fluence64 + idx, static_cast<double>(v));
        } else {  // 32-bit element offsets (idx >= 0 here)
            unsigned a = static_cast<unsigned>(idx);
            if (REP == kRepWhole) a += rep.base;
            if (REP == kRepPrefix) a += a < rep.len ? rep.base : 0u;
            atomicAdd(B.fluence64 + a, static_cast<double>(v));
        }
    } else {
        atomicAdd(B.fluence + idx, v);
    }
}

__global__ void k_fp64_to_fp32(const double* __restrict__ src, float* __restrict__ dst, unsigned long long n,
                               unsigned reps, unsigned long long len);

// =============================================================================================== loop building blocks
// Per-lane event counts.  The fast kernels do not count scatters one by one: there every voxel step either crosses
// a voxel boundary, uses up the free path (and the photon scatters) or stops the photon (step cap, zero-progress
// guard), so the scatters are steps - crossings - stopped photons (flush_tallies and rare_flush).  The strict kernels
// skip the step when the free path is 0, as the reference does (L283), so they count scatters in `scat`.
struct Counters {
    unsigned steps = 0, cross = 0, scat = 0;
};

// Per-CTA counts of rare events (photon launches, reflections, photons stopped by a guard), kept with shared-memory
// atomics so that they take no registers in the hot loop.  Every kernel resets them before its first barrier and
// adds them to the launch's statistics after its loop (rare_flush, reached by all threads).
enum { kRareLaunch = 0, kRareRefl = 1, kRareCap = 2 };
static __shared__ unsigned long long s_rare[3];
__device__ __forceinline__ void rare_reset() {
    if (threadIdx.x < 3) s_rare[threadIdx.x] = 0ULL;
}
__device__ __forceinline__ void rare_count(int k) { atomicAdd(&s_rare[k], 1ULL); }

// launch deadline of the CTA (wall clock, %globaltimer), set by thread 0 before the kernel's first barrier
static __shared__ unsigned long long s_tend;

// dynamic shared memory a propagation kernel's CTA can have next to the engine's static shared memory
// (the prefetched photon indices, the rare-event counts and the deadline), with room for alignment
constexpr size_t kMaxDynamicSmem = 227u * 1024u - (1024u * 8u + 3u * 8u + 8u) - 256u;
__device__ __forceinline__ void set_deadline(unsigned long long budget_ns) {
    if (threadIdx.x == 0) s_tend = global_ns() + budget_ns;
}

// what one loop iteration did to an active photon
struct Event {
    bool crossed;        // a voxel boundary was crossed: a deposit site (L285)
    bool term;           // the photon terminated
    bool scattered;      // a scattering event happened, in medium scat_mid
    int left_vox;        // voxel left at the crossing
    unsigned left_mid;   // its medium
    int gate;            // time gate of the deposit (negative before tstart)
    float seg;           // path since the previous deposit site (len.z before the reset)
    float w_before;      // weight at the previous deposit site (len.w before the reset)
    float dep_val;       // the value MCX_photon::save deposits (L360)
    unsigned scat_mid;
};

// Label source of the propagation loop: the uint8 volume read through the read-only path.
struct GlobalLabels {
    const uint8_t* __restrict__ p;
#if UMCX_DEVICE_CHECKS
    unsigned long long n;  // voxels of the volume
    unsigned nmedia;       // media of its table
    int* err;
#endif
    __device__ __forceinline__ unsigned operator()(int i) const {
#if UMCX_DEVICE_CHECKS
        if (!index_ok(err, static_cast<unsigned long long>(static_cast<long long>(i)), n, kSiteLabel)) return 0u;
        const unsigned v = __ldg(p + i);
        return index_ok(err, v & UMCX_LABEL_MASK, nmedia, kSiteMedium) ? v : 0u;
#else
        return __ldg(p + i);
#endif
    }
};
// label view of n voxels at byte offset off of the label buffer, naming nmedia media
__device__ __forceinline__ GlobalLabels global_labels(const KBuffers& B, unsigned long long off, unsigned long long n,
                                                      unsigned nmedia) {
    GlobalLabels g;
    g.p = B.labels + off;
#if UMCX_DEVICE_CHECKS
    g.n = off + n <= B.n_labels ? n : 0;  // a view that overruns the buffer fails its first read
    g.nmedia = nmedia;
    g.err = &B.stats->error;
#else
    (void)n;
    (void)nmedia;
#endif
    return g;
}

// the kernels call this where a photon ends: photons stopped by the step cap or the zero-progress guard (a photon
// that reaches either limit ends at that step, so the test here finds exactly those)
__device__ __forceinline__ void count_stopped(const Photon& p) {
    if (p.nsteps > kDefaultStepCap || p.media >= (kZeroStepLimit << 16)) rare_count(kRareCap);
}

// Boundary reflection switch of one simulation.  A single-simulation kernel is instantiated with REFLECT equal to
// its isreflect, so nothing is read at run time; a batch kernel with reflections reads each simulation's flag.
__device__ __forceinline__ bool reflect_on(const KParams&) { return true; }
template <class PV>
__device__ __forceinline__ bool reflect_on(const PV& S) { return S.isreflect != 0; }

template <bool STRICT, class PV>
__device__ __forceinline__ int deposit_gate(const PV& P, const Photon& p);  // (below)

// L761-762 + L262-271: seed photon idx, launch it, move it onto the grid; false when it misses the grid
template <bool STRICT, class PV, class LV>
__device__ __forceinline__ bool start_photon(const PV& P, const LV& labels, Photon& p, unsigned long long idx) {
    p.launchw = launch<STRICT>(P, p, idx);
    p.lastvox = vox_index(P, p.ix, p.iy, p.iz);
    const bool inside = p.lastvox >= 0 || skip_to_grid(P, p);
    if (inside) {
        p.media = labels(p.lastvox);
        p.lx = scat_len<STRICT>(p.rng);
    } else {
        p.media = 0;
    }
    return inside;
}

// One iteration for an active photon: a voxel step and, at a voxel change, the deposit bookkeeping, time-gate test,
// boundary handling and label update of MCX_photon::sprint (L281-314); then a scatter when the free path is used up
// (L272-274).  Every kernel (forward, adjoint, replay) advances photons with this one function, so a replayed photon
// follows the forward pass's trajectory.  RESET_SEGMENT resets the deposit segment at every crossing even when no
// volume is saved (per-voxel path lengths for the adjoint and the replay); trajectories do not depend on it.
// SAVEVOL as for photon_step.
template <bool STRICT, bool REFLECT, bool RESET_SEGMENT, int SAVEVOL = -1, class PV, class LV>
__device__ __forceinline__ void advance(const PV& P, const LV& labels, const Medium* sm, Photon& p, Event& ev,
                                        Counters& c, bool active = true) {
    ev.crossed = false;
    ev.term = false;
    ev.scattered = false;
    if (active && (!STRICT || p.lx > 0.f)) {  // a fast step with lx = 0 moves nothing (as in photon_step)
        const unsigned mid = p.media & UMCX_LABEL_MASK;
        const Medium m = sm[mid];
        bool crossed;
        float moved;
        int newvox = step<STRICT>(P, p, m, &crossed, &moved);
        c.steps++;
        // zero-progress guard: a direction component that is exactly zero at a grid face can make a photon alternate
        // forever between a zero-length crossing and a reflection that puts it back (the inverse direction is stale
        // after a launch or a refraction, as in the reference); count consecutive zero-length steps in bits 16+ of
        // `media` and stop the photon after kZeroStepLimit of them, like the step cap
        if (moved == 0.f) p.media += 0x10000u;
        else p.media &= 0xFFFFu;
        const bool capped = ++p.nsteps > kDefaultStepCap || p.media >= (kZeroStepLimit << 16);  // (count_stopped)
        ev.term = capped;
        if (!capped && newvox != p.lastvox) {
            c.cross++;
            ev.crossed = true;
            ev.left_vox = p.lastvox;
            ev.left_mid = mid;
            ev.seg = p.lz;
            ev.w_before = p.lw;
            ev.gate = deposit_gate<STRICT>(P, p);
            ev.dep_val = deposit_value<STRICT>(P, p, m);
            if (RESET_SEGMENT || (SAVEVOL < 0 ? P.issavevol != 0 : SAVEVOL != 0)) {
                p.lw = p.pw;
                p.lz = 0.f;
            }
            // past the last gate the photon ends here; otherwise the next voxel's label decides: leaving the grid
            // or tissue -> background ends it, a refractive-index change reflects or transmits it (L291-306)
            const bool late = p.ly > P.tend;
            unsigned newmedia = (newvox >= 0 && !late) ? labels(newvox) : 0u;
            const float n2 = sm[newmedia & UMCX_LABEL_MASK].a.w;
            bool term = late || newvox < 0 || ((newmedia & UMCX_LABEL_MASK) == 0 && mid != 0);
            if (REFLECT && reflect_on(P) && !late && m.a.w != n2) {
                rare_count(kRareRefl);
                if (reflect<STRICT>(p, m.a.w, n2)) {
                    term = newvox < 0 || (newmedia & UMCX_LABEL_MASK) == 0;
                } else {
                    term = false;
                    newvox = p.lastvox;
                    newmedia = p.media;
                }
            }
            ev.term = term;
            if (!term) {
                p.lastvox = newvox;
                p.media = newmedia;
            }
        }
    }
    if (active && !ev.term && p.lx <= 0.f) {
        ev.scattered = true;
        ev.scat_mid = p.media & UMCX_LABEL_MASK;
        scatter<STRICT>(p, sm[ev.scat_mid]);
        if (STRICT) c.scat++;
    }
}

// per-lane photon indices: the first is the lane's global index, the next one is fetched from the global counter
// when the current one starts, so the atomic's latency overlaps the photon's whole life
// (indices [0, lanes) are the lanes' first photons; counter value c stands for photon lanes + c).  The prefetched
// index is touched once per photon and lives in shared memory, not in the hot loop's registers.
static __shared__ unsigned long long s_next[1024];
struct PhotonFeed {
    __device__ __forceinline__ void init(unsigned long long* counter, unsigned long long gid, unsigned long long total,
                                         unsigned long long lanes) {
        (void)counter;
        (void)total;
        (void)lanes;
        s_next[threadIdx.x] = gid;
    }
    // false when no photon is left; otherwise returns the prefetched index and prefetches the following one
    __device__ __forceinline__ bool take(unsigned long long* counter, unsigned long long* idx, unsigned long long n) {
        const unsigned long long next = s_next[threadIdx.x];
        if (next >= n) return false;
        *idx = next;
        s_next[threadIdx.x] = atomicAdd(counter, 1ULL) + static_cast<unsigned long long>(gridDim.x) * blockDim.x;
        return true;
    }
};

__device__ __forceinline__ bool det_hit(const float4 dp, const Photon& p) {  // L430-431
    return (dp.x - p.px) * (dp.x - p.px) + (dp.y - p.py) * (dp.y - p.py) + (dp.z - p.pz) * (dp.z - p.pz) < dp.w * dp.w;
}

// fluence deposit of one iteration, called by all lanes of the warp (converged)
template <int REP = kRepNone>
__device__ __forceinline__ void deposit_converged(const KBuffers& B, bool aggregate, float* aggbuf, unsigned tid,
                                                  unsigned lane, int dep_idx, float dep_val,
                                                  Replica rep = Replica{0u, 0u}) {
    if (aggregate) {
        const unsigned hm = __ballot_sync(kFull, dep_idx >= 0);
        if (__popc(hm) > 1) {
            const unsigned grp = __match_any_sync(kFull, dep_idx >= 0 ? static_cast<unsigned>(dep_idx) : 0xFFFFFFFFu);
            aggbuf[tid] = dep_val;
            __syncwarp();
            if (dep_idx >= 0 && lane == __ffs(grp) - 1u) {
                float s = 0.f;
                const unsigned base = tid & ~31u;
                for (unsigned g = grp; g; g &= g - 1) s += aggbuf[base + __ffs(g) - 1];
                deposit_add<REP>(B, dep_idx, s, rep);
            }
            __syncwarp();
            return;
        }
    }
    if (dep_idx >= 0) deposit_add<REP>(B, dep_idx, dep_val, rep);
}

// Detected-photon append (L276-278, L429-435; MCX_detect::addphoton L164-176), called only by the lanes of a warp
// that end a photon in this iteration (no vote runs in the other iterations).  Among those lanes, per detector: a
// ballot of the hits, one atomic per warp for the block of slots, and each hit's slot from a prefix count of the
// ballot.  write(d, slot) stores the record of a slot below the buffer size; all hits are counted.
template <class WriteRecord>
__device__ __forceinline__ void append_detected(const KParams& P, const KBuffers& B, unsigned lane, bool tdet,
                                                const Photon& p, WriteRecord&& write) {
    const unsigned group = __activemask();
    if (!__any_sync(group, tdet)) return;
    const unsigned below = (1u << lane) - 1u;
    for (int d = 0; d < P.detnum; d++) {
        const bool hit = tdet && det_hit(P.det[d], p);
        const unsigned hm = __ballot_sync(group, hit);
        if (hm == 0u) continue;
        const unsigned leader = __ffs(hm) - 1u;
        unsigned long long base = 0;
        if (lane == leader) base = atomicAdd(&B.stats->detected, static_cast<unsigned long long>(__popc(hm)));
        base = __shfl_sync(group, base, leader);
        if (hit) {
            const unsigned long long slot = base + __popc(hm & below);
            if (slot < P.maxdetphotons) write(d, slot);
        }
    }
}

// the standard record of L171-174: [detid][ppath x ppathlen][exit position][exit direction], in row `slot` of the
// record array that starts `base` floats into B.detp (0 for a single simulation; the simulation's offset in a batch)
template <class PV>
__device__ __forceinline__ void write_detp(const PV& P, const KBuffers& B, const Photon& p, const float* ppath,
                                           unsigned stride, int d, unsigned long long slot,
                                           unsigned long long base = 0) {
    if (!index_ok(&B.stats->error, base + (slot + 1) * static_cast<unsigned long long>(P.cols),
                  UMCX_EXTENT(B, n_detp) + 1, kSiteDetRow))
        return;
    float* rec = B.detp + base + slot * static_cast<unsigned long long>(P.cols);
    int k = 0;
    if (P.savedetflag & UMCX_DET_ID) rec[k++] = static_cast<float>(d + 1);
    if (P.savedetflag & UMCX_DET_PPATH)
        for (int q = 0; q < P.ppathlen; q++) rec[k++] = ppath[q * stride];
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

// per-warp reduction of the lane tallies, one set of atomics per warp
template <bool STRICT = false>
__device__ __forceinline__ void flush_tallies(const KBuffers& B, unsigned lane, double tot, double esc, Counters c) {
    for (int off = 16; off > 0; off >>= 1) {
        tot += __shfl_down_sync(kFull, tot, off);
        esc += __shfl_down_sync(kFull, esc, off);
        c.steps += __shfl_down_sync(kFull, c.steps, off);
        c.cross += __shfl_down_sync(kFull, c.cross, off);
        if (STRICT) c.scat += __shfl_down_sync(kFull, c.scat, off);
    }
    if (lane == 0) {
        atomicAdd(&B.stats->total, tot);
        atomicAdd(&B.stats->escape, esc);
        atomicAdd(&B.stats->steps, static_cast<unsigned long long>(c.steps));
        atomicAdd(&B.stats->crossings, static_cast<unsigned long long>(c.cross));
        // fast kernels: steps - crossings (the CTA's stopped photons are taken off in rare_flush); modulo 2^64, so the
        // total is exact whenever every photon ended (a launch stopped by its wall-clock budget reports partial counts)
        atomicAdd(&B.stats->scatters, STRICT ? static_cast<unsigned long long>(c.scat)
                                             : static_cast<unsigned long long>(c.steps) - c.cross);
    }
}

// the CTA's rare-event counts into the launch statistics; every thread of the CTA must call it
template <bool STRICT = false>
__device__ __forceinline__ void rare_flush(const KBuffers& B) {
    __syncthreads();
    if (threadIdx.x == 0) {
        atomicAdd(&B.stats->launched, s_rare[kRareLaunch]);
        atomicAdd(&B.stats->reflections, s_rare[kRareRefl]);
        if (s_rare[kRareCap]) {
            atomicAdd(&B.stats->capped, s_rare[kRareCap]);
            if (!STRICT) atomicAdd(&B.stats->scatters, 0ULL - s_rare[kRareCap]);  // its last step did not scatter
        }
    }
}

// copies the media table (3 float4 per medium) into shared memory
__device__ __forceinline__ void load_media(const KParams& P, const Medium* src, Medium* sm) {
    rare_reset();
    set_deadline(P.budget_ns);
    const float4* s = reinterpret_cast<const float4*>(src);
    float4* d = reinterpret_cast<float4*>(sm);
    for (int k = threadIdx.x; k < 3 * P.mediumnum; k += blockDim.x) d[k] = s[k];
    __syncthreads();
}

// uniform exit of a warp when the launch's wall-clock budget (deadline s_tend) is used up
__device__ __forceinline__ bool out_of_budget(const KBuffers& B, unsigned iter, unsigned lane) {
    if ((iter & 1023u) != 0u) return false;
    const bool late = global_ns() > s_tend;
    if (__any_sync(kFull, late)) {
        if (lane == 0) atomicExch(&B.stats->error, UMCX_ERR_TIMEOUT);
        return true;
    }
    return false;
}

// One iteration for an active photon: a voxel step and, at a voxel change, the bookkeeping, time-gate test, boundary
// handling and label update of MCX_photon::sprint (L281-314); then a scatter when the free path is used up
// (L272-274).  What a kernel records is done in place by two callbacks -- at a crossing, on_cross(mid, m) with the
// photon still holding the segment just ended (p.lz: path since the last deposit, p.lw: weight there, p.pw: weight
// now, p.lastvox: the voxel left, of medium mid), and after a scatter in medium mid, on_scatter(mid) -- so that
// nothing a crossing records stays live through the scattering code.  Returns true when the photon ended.
// RESET_SEGMENT resets the deposit segment at every crossing even when no volume is saved (per-voxel path lengths
// for the adjoint and the replay); trajectories do not depend on it.  SAVEVOL as for record_crossing (whether the
// volume is saved: 1 / 0 known at compile time, -1 read from P).  Every kernel advances photons with this
// function (the warp-aggregated forward and batched instances with advance(), which performs the same operations
// in the same order), so a replayed photon follows the forward pass's trajectory.
// PV is KParams (a single simulation) or SimDesc (a simulation of a batch).
template <bool STRICT, bool REFLECT, bool RESET_SEGMENT, int SAVEVOL = -1, class PV, class LV, class OnCross,
          class OnScatter>
__device__ __forceinline__ bool photon_step(const PV& P, const LV& labels, const Medium* sm, Photon& p, Counters& c,
                                            OnCross&& on_cross, OnScatter&& on_scatter) {
    bool term = false;
    // the reference steps only while lx > 0 (L283); a fast step with lx = 0 moves nothing and does not cross, so the
    // fast kernels skip the test (the scatter below follows in both cases; only the step count differs)
    if (!STRICT || p.lx > 0.f) {
        const unsigned mid = p.media & UMCX_LABEL_MASK;
        const Medium m = sm[mid];
        bool crossed;
        float moved;
        int newvox = step<STRICT>(P, p, m, &crossed, &moved);
        // (the lane's step count is taken from p.nsteps when the photon ends)
        // zero-progress guard and step cap, as in advance()
        if (moved == 0.f) p.media += 0x10000u;
        else p.media &= 0xFFFFu;
        const bool capped = ++p.nsteps > kDefaultStepCap || p.media >= (kZeroStepLimit << 16);
        term = capped;
        if (!capped && newvox != p.lastvox) {
            c.cross++;
            // the next voxel's label first: its load overlaps the recording below
            const bool late = p.ly > P.tend;
            unsigned newmedia = (newvox >= 0 && !late) ? labels(newvox) : 0u;
            on_cross(mid, m);
            if (RESET_SEGMENT || (SAVEVOL < 0 ? P.issavevol != 0 : SAVEVOL != 0)) {
                p.lw = p.pw;
                p.lz = 0.f;
            }
            const float n2 = sm[newmedia & UMCX_LABEL_MASK].a.w;
            term = late || newvox < 0 || ((newmedia & UMCX_LABEL_MASK) == 0 && mid != 0);
            if (REFLECT && reflect_on(P) && !late && m.a.w != n2) {
                rare_count(kRareRefl);
                if (reflect<STRICT>(p, m.a.w, n2)) {
                    term = newvox < 0 || (newmedia & UMCX_LABEL_MASK) == 0;
                } else {
                    term = false;
                    newvox = p.lastvox;
                    newmedia = p.media;
                }
            }
            if (!term) {
                p.lastvox = newvox;
                p.media = newmedia;
            }
        }
    }
    if (!term && p.lx <= 0.f) {
        const unsigned mid = p.media & UMCX_LABEL_MASK;
        scatter<STRICT>(p, sm[mid]);
        if (STRICT) c.scat++;
        on_scatter(mid);
    }
    return term;
}

// x = (t - tstart) * rtstep, the position of time t in the gates (L290).  The fast kernels of a single simulation
// compute it as one fused multiply-add t * rtstep + gate_off (gate_off = -tstart * rtstep), identical when tstart is
// 0 and within a rounding of it otherwise; the strict kernels and a batch's simulations use the reference's form.
template <bool STRICT, class PV>
__device__ __forceinline__ float gate_pos(const PV& P, float t) {
    return (t - P.tstart) * P.rtstep;
}
template <bool STRICT>
__device__ __forceinline__ float gate_pos(const KParams& P, float t) {
    if constexpr (STRICT) return (t - P.tstart) * P.rtstep;
    else return fmaf(t, P.rtstep, P.gate_off);
}

// the time gate of a deposit at the photon's current time: (int)fminf(maxgate - 1, floorf(x)) as one rounding
// conversion and an integer min (same value for every x: the conversion saturates like the reference's cast chain
// does on the device); negative before tstart
template <bool STRICT, class PV>
__device__ __forceinline__ int deposit_gate(const PV& P, const Photon& p) {
    return min(__float2int_rd(gate_pos<STRICT>(P, p.ly)), P.maxgate - 1);
}

// the forward kernels' crossing record: partial path of the medium left (L286-288) and the fluence deposit
// (L289-291, L359-363) through deposit(voxel, gate, value).  SAVEVOL: 1 / 0 when the launch is known to save / not
// to save the output volume, -1 to read P.issavevol.  The partial-path test is one unsigned compare: ppathlen is 0
// unless partial paths are saved, and label 0 (mid - 1 wraps) has no column.  GATE1: the volume has one time gate,
// so deposit_gate is 0 exactly when (t - tstart) * rtstep >= 0 and negative otherwise (for every time that is not
// NaN), which is all the crossing needs to know.
template <bool STRICT, bool SAVEDET, int SAVEVOL = -1, bool GATE1 = false, class PV, class Deposit>
__device__ __forceinline__ void record_crossing(const PV& P, const Photon& p, unsigned mid, const Medium& m,
                                                float* ppath_lane, int* err, Deposit&& deposit) {
    (void)err;
    if constexpr (SAVEDET) {
        if (mid - 1u < static_cast<unsigned>(P.ppathlen)) ppath_lane[(mid - 1) * blockDim.x] += p.lz;
    }
    if (SAVEVOL < 0 ? P.issavevol != 0 : SAVEVOL != 0) {
        if constexpr (GATE1) {
            if (gate_pos<STRICT>(P, p.ly) >= 0.f) deposit(p.lastvox, 0, deposit_value<STRICT>(P, p, m));
        } else {
            const int gate = deposit_gate<STRICT>(P, p);
            if (gate >= 0) deposit(p.lastvox, gate, deposit_value<STRICT>(P, p, m));
        }
    }
}

// =============================================================================================== forward kernel
// Shared memory: double tally[2][blockDim] | Medium[mediumnum] | float ppath[ppathlen][blockDim] |
// float aggbuf[blockDim] | float launch weight[blockDim]
// launch bounds of the forward kernel (a build variant can trade resident lanes for registers, e.g.
// UMCX_NVCC_DEFS="UMCX_FWD_THREADS=256 UMCX_FWD_MINB=3"; measured on GB300 the default 1024 x 1 at 64 registers is
// as fast as 768 lanes at 74 registers and faster than 512 lanes at 86)
#ifndef UMCX_FWD_THREADS
#define UMCX_FWD_THREADS 1024
#define UMCX_FWD_MINB 1
#endif
// REP: replication mode of the FP64 output volume (P.rep_mask, P.rep_len; see accumulator_replicas); AGG: fluence
// deposits aggregated per warp with __match_any_sync (P.aggregate) instead of plain atomics; GATE1: the output volume
// has one time gate (plain-atomic instances)
template <bool STRICT, bool REFLECT, bool SAVEDET, int REP = kRepNone, bool AGG = false, bool GATE1 = false>
__global__ void __launch_bounds__(UMCX_FWD_THREADS, UMCX_FWD_MINB) k_forward(const KParams P, const KBuffers B) {
    extern __shared__ float4 smem4[];
    // per-lane FP64 energy tallies and launch weight live in shared memory (touched once per photon), which keeps
    // them out of the register budget of the hot loop
    double* tally = reinterpret_cast<double*>(smem4);  // [2][blockDim]: total, escape
    Medium* sm = reinterpret_cast<Medium*>(tally + 2 * blockDim.x);
    float* ppath = reinterpret_cast<float*>(sm + P.mediumnum);
    float* aggbuf = ppath + (SAVEDET ? P.ppathlen * blockDim.x : 0);
    float* lwbuf = aggbuf + blockDim.x;
    const GlobalLabels labels = global_labels(B, 0, P.dimxyz, static_cast<unsigned>(P.mediumnum));
    load_media(P, B.media, sm);

    const unsigned tid = threadIdx.x;
    const unsigned lane = lane_id();
    tally[tid] = 0.0;
    tally[blockDim.x + tid] = 0.0;
    PhotonFeed feed;
    feed.init(B.counter, static_cast<unsigned long long>(blockIdx.x) * blockDim.x + tid, P.nphoton,
              static_cast<unsigned long long>(gridDim.x) * blockDim.x);
    Photon p;
    p.media = 0;
    p.lastvox = -1;
    bool active = false, done = false;
    Counters c;
    const Replica replica = cta_replica<REP>(P);
    constexpr int SAVEVOL = REP == kRepOff ? 0 : 1;  // kRepOff: the launch saves no output volume

    for (unsigned iter = 0;; iter++) {
        if (!active && !done) {  // launch a photon on an idle lane (L761-763)
            unsigned long long k;
            if (!feed.take(B.counter, &k, P.nphoton)) {
                done = true;
            } else {
                rare_count(kRareLaunch);
                active = start_photon<STRICT>(P, labels, p, P.photon_offset + k);
                lwbuf[tid] = p.launchw;
                if (SAVEDET && active)
                    for (int q = 0; q < P.ppathlen; q++) ppath[q * blockDim.x + tid] = 0.f;
            }
        }
        // warp-uniform exits, tested every 16 iterations (a finished lane idles for at most 15 more)
        if ((iter & 15u) == 0u) {
            if (__all_sync(kFull, done)) break;
            if (out_of_budget(B, iter, lane)) break;
        }

        bool term = false;
        if (AGG) {
            Event ev;
            advance<STRICT, REFLECT, false, SAVEVOL>(P, labels, sm, p, ev, c, active);  // no event on an idle lane
            if (SAVEDET && ev.crossed && ev.left_mid - 1u < static_cast<unsigned>(P.ppathlen))
                ppath[(ev.left_mid - 1) * blockDim.x + tid] += ev.seg;  // L286-288
            const bool dep = SAVEVOL && ev.crossed && ev.gate >= 0;
            const int dep_idx = dep ? ev.left_vox + ev.gate * static_cast<int>(P.dimxyz) : -1;
            const float dep_val = dep ? ev.dep_val : 0.f;
            deposit_converged<REP>(B, true, aggbuf, tid, lane, dep_idx, dep_val, replica);
            term = ev.term;
        } else if (active) {
            term = photon_step<STRICT, REFLECT, false, SAVEVOL>(
                P, labels, sm, p, c,
                [&](unsigned mid, const Medium& m) {
                    record_crossing<STRICT, SAVEDET, SAVEVOL, GATE1>(P, p, mid, m, ppath + tid, &B.stats->error,
                                                     [&](int vox, int gate, float v) {
                                                         deposit_add<REP>(B, vox + gate * static_cast<int>(P.dimxyz), v,
                                                                          replica);
                                                     });
                },
                [](unsigned) {});
        }
        if (term) {
            count_stopped(p);
            if (!AGG) c.steps += p.nsteps;  // photon_step does not count steps one by one
            if (SAVEDET) {
                const bool tdet = (p.media & UMCX_LABEL_DET) && p.ly <= P.tend;
                append_detected(P, B, lane, tdet, p, [&](int d, unsigned long long slot) {
                    write_detp(P, B, p, ppath + tid, blockDim.x, d, slot);
                });
            }
            if ((p.media & UMCX_LABEL_MASK) != 0u) {  // energy tallies (L765-770)
                tally[tid] += static_cast<double>(lwbuf[tid]);
                tally[blockDim.x + tid] += static_cast<double>(p.pw);
            }
            active = false;
        }
    }
    flush_tallies<STRICT>(B, lane, tally[tid], tally[blockDim.x + tid], c);
    rare_flush<STRICT>(B);
}

// =============================================================================================== adjoint kernel
// The forward pass of the adjoint: the forward kernel's outputs plus, per photon, the tallies that make the
// derivatives of the summed output volume with respect to every label's mua and mus, and an extended record per
// detected photon (photon index, detector, exit weight and time, path and scatter count per label).
//
// Fluence derivatives (F_j = deposit j, in label m_j, segment length l_j, L_k(<j) / n_k(<=j) = path / scatters in
// label k before deposit j, S = running sum of F):
//   dSum/dmua_k = -sum_j L_k(<j) F_j + sum_{j: m_j = k} dF_j/dmua_k|path
//               = -(L_k S - Q_k) + E_k            with Q_k += l_j S (after adding F_j), E_k += dF_j/dmua
//   dSum/dmus_k = sum_j F_j (n_k(<=j)/mus_k - L_k(<=j))           (score of the path prefix up to deposit j)
//               = (cnt_k S - R_k)/mus_k - (L_k S - Q_k + T_k)   with R_k += S at each scatter, T_k += F_j l_j
// so each deposit and each scatter updates one label's tallies (O(1) per event).
//
// Shared memory: double ga[K], gs[K], total, escape | Medium[K] | float ppath[ppathlen][bd] |
// float L, cnt, Q, T, E, R[K][bd] | u64 photon index[bd]
// REP: replication mode of the FP64 output volume, as in the forward kernel
template <bool REFLECT, int REP = kRepNone>
__global__ void __launch_bounds__(1024) k_adjoint(const KParams P, const KBuffers B) {
    extern __shared__ double smem8[];
    const unsigned bd = blockDim.x;
    const int K = P.mediumnum;
    // the CTA's FP64 accumulators of the per-label gradients and of the energy tallies, added to with shared-memory
    // atomics once per photon (per-lane copies would take shared memory from the L1 that caches the labels)
    double* ga = smem8;   // [K]
    double* gs = ga + K;  // [K]
    double* et = gs + K;  // [2]: total, escape
    Medium* sm = reinterpret_cast<Medium*>(et + 2);
    float* ppath = reinterpret_cast<float*>(sm + K);
    float* Lk = ppath + P.ppathlen * bd;
    float* Ck = Lk + K * bd;
    float* Qk = Ck + K * bd;
    float* Tk = Qk + K * bd;
    float* Ek = Tk + K * bd;
    float* Rk = Ek + K * bd;
    // touched once per photon, so kept out of the loop's registers: the photon index
    unsigned long long* cur = reinterpret_cast<unsigned long long*>(Rk + K * bd);  // [bd]
    // the label view is built from kernel parameters where it is used, so it holds no registers in the loop
    auto labels = [&]() { return global_labels(B, 0, P.dimxyz, static_cast<unsigned>(P.mediumnum)); };
    for (int k = threadIdx.x; k < 2 * K + 2; k += bd) ga[k] = 0.0;
    load_media(P, B.media, sm);

    const unsigned tid = threadIdx.x;
    const unsigned lane = lane_id();
    PhotonFeed feed;
    feed.init(B.counter, static_cast<unsigned long long>(blockIdx.x) * bd + tid, P.nphoton,
              static_cast<unsigned long long>(gridDim.x) * bd);
    Photon p;
    p.media = 0;
    p.lastvox = -1;
    bool active = false, done = false;
    cur[tid] = 0;
    Counters c;
    float S = 0.f;
    const Replica replica = cta_replica<REP>(P);

    for (unsigned iter = 0;; iter++) {
        if (!active && !done) {
            unsigned long long k;
            if (!feed.take(B.counter, &k, P.nphoton)) {
                done = true;
            } else {
                rare_count(kRareLaunch);
                cur[tid] = P.photon_offset + k;
                active = start_photon<false>(P, labels(), p, P.photon_offset + k);
                if (active) {
                    S = 0.f;
                    for (int q = 0; q < P.ppathlen; q++) ppath[q * bd + tid] = 0.f;
                    for (int q = 0; q < K; q++) {
                        Lk[q * bd + tid] = 0.f;
                        Ck[q * bd + tid] = 0.f;
                        Qk[q * bd + tid] = 0.f;
                        Tk[q * bd + tid] = 0.f;
                        Ek[q * bd + tid] = 0.f;
                        Rk[q * bd + tid] = 0.f;
                    }
                }
            }
        }
        // warp-uniform exits, tested every 16 iterations (a finished lane idles for at most 15 more)
        if ((iter & 15u) == 0u) {
            if (__all_sync(kFull, done)) break;
            if (out_of_budget(B, iter, lane)) break;
        }

        bool term = false;
        if (active) {
            term = photon_step<false, REFLECT, true>(
                P, labels(), sm, p, c,
                [&](unsigned m, const Medium& med) {
                    const float seg = p.lz;  // path in the voxel left (the segment is reset at every crossing)
                    if (m - 1u < static_cast<unsigned>(P.ppathlen)) ppath[(m - 1) * bd + tid] += seg;
                    float F = 0.f, dF = 0.f;
                    if (P.issavevol) {
                        const int gate = deposit_gate<false>(P, p);
                        if (gate >= 0) {
                            F = deposit_value<false>(P, p, med);
                            deposit_add<REP>(B, p.lastvox + gate * static_cast<int>(P.dimxyz), F, replica);
                            // derivative of this deposit with respect to its own label's mua along the fixed path
                            if (P.outputtype == UMCX_OUT_ENERGY) {
                                dF = seg * p.pw;  // d(w0 (1 - e^-mua l))/dmua = l w1
                            } else {
                                // fluence = integral of w over the segment; derivative -w0 (1 - (1 + x) e^-x) / mua^2,
                                // x = mua l, by its series for small x (also the mua -> 0 limit -w0 l^2 / 2)
                                const float mua = med.a.x;
                                const float x = mua * seg;
                                float i1;
                                if (x < 0.1f) {
                                    i1 = seg * seg *
                                         (0.5f + x * (-1.f / 3.f + x * (0.125f + x * (-1.f / 30.f + x * (1.f / 144.f)))));
                                } else {
                                    i1 = (1.f - (1.f + x) * expf(-x)) / (mua * mua);
                                }
                                dF = -p.lw * i1;
                            }
                        }
                    }
                    S += F;
                    Lk[m * bd + tid] += seg;
                    Qk[m * bd + tid] += seg * S;
                    Tk[m * bd + tid] += F * seg;
                    Ek[m * bd + tid] += dF;
                },
                [&](unsigned m) {
                    Ck[m * bd + tid] += 1.f;
                    Rk[m * bd + tid] += S;
                });
        }
        if (term) {
            count_stopped(p);
            c.steps += p.nsteps;  // photon_step does not count steps one by one
            // detection (L429-435): the terminating lane appends its records, one atomic per detector hit, with
            // the extended record (photon index, exit weight and time, per-label path and scatter counts)
            const bool tdet = (p.media & UMCX_LABEL_DET) && p.ly <= P.tend;
            append_detected(P, B, lane, tdet, p, [&](int d, unsigned long long slot) {
                if (B.detp) write_detp(P, B, p, ppath + tid, bd, d, slot);
                DetRecord r;
                r.photon = cur[tid];
                r.det = d + 1;
                r.weight = p.pw;
                r.time = p.ly;
                r.pad = 0.f;
                B.detrec[slot] = r;
                float* ext = B.detext + slot * static_cast<unsigned long long>(2 * K);
                for (int q = 0; q < K; q++) {
                    ext[q] = Lk[q * bd + tid];
                    ext[K + q] = Ck[q * bd + tid];
                }
            });
            if ((p.media & UMCX_LABEL_MASK) != 0u) {
                atomicAdd(et, static_cast<double>(p.launchw));
                atomicAdd(et + 1, static_cast<double>(p.pw));
            }
            for (int q = 0; q < K; q++) {
                const float L = Lk[q * bd + tid];
                const float lsq = L * S - Qk[q * bd + tid];
                atomicAdd(ga + q, static_cast<double>(-lsq + Ek[q * bd + tid]));
                const float mus = sm[q].a.y;
                const float a = Ck[q * bd + tid] * S - Rk[q * bd + tid];
                atomicAdd(gs + q, static_cast<double>((mus > 0.f ? a / mus : 0.f) - (lsq + Tk[q * bd + tid])));
            }
            active = false;
        }
    }
    flush_tallies(B, lane, 0.0, 0.0, c);
    rare_flush(B);  // (its barrier also orders every lane's accumulator updates before the reads below)
    if (threadIdx.x == 0) {
        atomicAdd(&B.stats->total, et[0]);
        atomicAdd(&B.stats->escape, et[1]);
        for (int q = 0; q < K; q++) {
            atomicAdd(B.grad + q, ga[q]);
            atomicAdd(B.grad + K + q, gs[q]);
        }
    }
}

// =============================================================================================== replay kernel
// Regenerates each recorded detected photon from its index (its RNG seed) and accumulates -w_exit * l into the
// voxel-wise mua Jacobian of its detector at every voxel it leaves (l = path inside that voxel).  The exit weight
// and detector of the replayed photon are compared with the record; differences are counted.
template <bool REFLECT>
__global__ void __launch_bounds__(1024) k_replay(const KParams P, const KBuffers B) {
    extern __shared__ float4 smem4[];
    Medium* sm = reinterpret_cast<Medium*>(smem4);
    load_media(P, B.media, sm);
    const unsigned lane = lane_id();
    PhotonFeed feed;
    feed.init(B.counter, static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x, B.replay_count,
              static_cast<unsigned long long>(gridDim.x) * blockDim.x);
    Photon p;
    p.media = 0;
    p.lastvox = -1;
    bool active = false, done = false;
    Counters c;
    DetRecord rec;
    rec.det = 0;
    rec.weight = 0.f;
    unsigned mismatch = 0;
    for (unsigned iter = 0;; iter++) {
        if (!active && !done) {
            unsigned long long k;
            if (!feed.take(B.counter, &k, B.replay_count)) {
                done = true;
            } else {
                rec = B.replay_list[k];
                rare_count(kRareLaunch);
                active = start_photon<false>(P, global_labels(B, 0, P.dimxyz, static_cast<unsigned>(P.mediumnum)), p,
                                             rec.photon);
                if (!active) mismatch++;
            }
        }
        // warp-uniform exits, tested every 16 iterations (a finished lane idles for at most 15 more)
        if ((iter & 15u) == 0u) {
            if (__all_sync(kFull, done)) break;
            if (out_of_budget(B, iter, lane)) break;
        }
        if (active) {
            const bool term = photon_step<false, REFLECT, true>(
                P, global_labels(B, 0, P.dimxyz, static_cast<unsigned>(P.mediumnum)), sm, p, c,
                [&](unsigned, const Medium&) {
                    const unsigned long long jidx = static_cast<unsigned long long>(rec.det - 1) * P.dimxyz + p.lastvox;
                    if (index_ok(&B.stats->error, jidx, UMCX_EXTENT(B, n_jacobian), kSiteJacobian))
                        atomicAdd(B.jacobian + jidx, -rec.weight * p.lz);
                },
                [](unsigned) {});
            if (term) {
                count_stopped(p);
                c.steps += p.nsteps;
                const bool same = (p.media & UMCX_LABEL_DET) && p.ly <= P.tend && det_hit(P.det[rec.det - 1], p) &&
                                  p.pw == rec.weight;
                if (!same) mismatch++;
                active = false;
            }
        }
    }
    for (int off = 16; off > 0; off >>= 1) mismatch += __shfl_down_sync(kFull, mismatch, off);
    if (lane == 0 && mismatch) atomicAdd(&B.stats->capped, static_cast<unsigned long long>(mismatch));
    flush_tallies(B, lane, 0.0, 0.0, c);
    rare_flush(B);
}

// =============================================================================================== batched kernel
// One simulation of a batch (224 bytes, staged in shared memory).  Member names match KParams so the engine
// functions (launch, step, advance, write_detp, ...) take either.
struct SimDesc {
    int nx, ny, nz, maxgate;
    unsigned dimyz, dimxyz;
    int isreflect, issavevol, outputtype, srctype;
    unsigned det_base, media_base;  // first detector / Medium of this simulation in the batch's tables
    float tstart, tend, rtstep, unitinmm;
    unsigned seeds[4];
    unsigned long long label_off;      // byte offset of its labels in the label pool
    unsigned long long out_off;        // element offset of its output volume in the output pool
    unsigned long long photon_offset;  // photon index of its first photon (seeds photon i as in a single run)
    unsigned long long nphoton;
    float4 srcpos, srcdir, srcrdir, srcparam1, srcparam2;
    // detected-photon records (L164-176, L429-435); detnum is 0 for a simulation that saves none
    int detnum, savedetflag, ppathlen, cols;
    unsigned long long maxdetphotons;  // rows reserved for it in the record pool
    unsigned long long detp_off;       // float offset of its first row in the record pool
};
static_assert(sizeof(SimDesc) == 224, "SimDesc layout");

struct BParams {
    const SimDesc* sims;              // [nsim]
    const unsigned long long* begin;  // [nsim + 1]: prefix sums of photon counts (batch photon index space)
    double* tallies;                  // [nsim][2]: escape, total (L765-770) per simulation
    const float4* dets;               // [total_det]: detectors {x, y, z, r} of the simulations that save records
    unsigned long long* detected;     // [nsim]: detections per simulation, including those beyond its row capacity
    int nsim, total_media, aggregate, total_det;
    int ppathlen;                     // largest ppathlen of the simulations (per-lane partial-path slots)
    int savedet;                      // some simulation saves detected photons: the SAVEDET instance runs
    unsigned long long total;         // photons in the whole batch
    unsigned long long budget_ns;
};

__device__ __forceinline__ void deposit_add64(const KBuffers& B, long long idx, float v) {
    if (!index_ok(&B.stats->error, static_cast<unsigned long long>(idx), UMCX_EXTENT(B, n_out), kSiteOutput)) return;
    if (B.fluence64) atomicAdd(B.fluence64 + idx, static_cast<double>(v));
    else atomicAdd(B.fluence + idx, v);
}

// Many independent simulations (different grids, label counts, optics, sources and photon budgets) in one
// persistent launch.  Lanes draw photon indices from one counter over the concatenated photon ranges; a binary
// search over the prefix sums names the simulation, whose descriptor and optical table sit in shared memory.
// Consecutive indices belong to the same simulation, so at any moment only one or two simulations are in flight and
// their outputs stay in L2, while the tail of one simulation overlaps the start of the next.
// SAVEDET: detected-photon records of the simulations that save them (a detection takes its row with one atomic on
// the simulation's counter: lanes of one warp can end photons of different simulations, and detections are rare).
// Shared memory: SimDesc[nsim] | u64 begin[nsim + 1] (padded to 16 B) | Medium[total_media] | float4 det[total_det] |
// float aggbuf[blockDim] | double escape, total[blockDim] | float ppath[ppathlen][blockDim]
template <bool REFLECT, bool AGG = false, bool SAVEDET = false>
__global__ void __launch_bounds__(1024) k_batch(const BParams BP, const KBuffers B) {
    extern __shared__ float4 smem4[];
    SimDesc* sd = reinterpret_cast<SimDesc*>(smem4);
    unsigned long long* begin = reinterpret_cast<unsigned long long*>(sd + BP.nsim);
    Medium* sm = reinterpret_cast<Medium*>(begin + ((BP.nsim + 2) & ~1));
    float4* sdet = reinterpret_cast<float4*>(sm + BP.total_media);
    float* aggbuf = reinterpret_cast<float*>(sdet + (SAVEDET ? BP.total_det : 0));
    double* etally = reinterpret_cast<double*>(aggbuf + blockDim.x);  // [2][blockDim]: escape, total of `tally_sim`
    float* ppath = reinterpret_cast<float*>(etally + 2 * blockDim.x);  // [ppathlen][blockDim] (SAVEDET)
    {
        constexpr int kDescVec = sizeof(SimDesc) / sizeof(float4);
        const float4* s = reinterpret_cast<const float4*>(BP.sims);
        float4* d = reinterpret_cast<float4*>(sd);
        for (int k = threadIdx.x; k < BP.nsim * kDescVec; k += blockDim.x) d[k] = s[k];
        for (int k = threadIdx.x; k <= BP.nsim; k += blockDim.x) begin[k] = BP.begin[k];
        const float4* ms = reinterpret_cast<const float4*>(B.media);
        float4* md = reinterpret_cast<float4*>(sm);
        for (int k = threadIdx.x; k < 3 * BP.total_media; k += blockDim.x) md[k] = ms[k];
        if (SAVEDET)
            for (int k = threadIdx.x; k < BP.total_det; k += blockDim.x) sdet[k] = BP.dets[k];
    }
    rare_reset();
    set_deadline(BP.budget_ns);
    __syncthreads();

    const unsigned tid = threadIdx.x;
    const unsigned lane = lane_id();
    PhotonFeed feed;
    feed.init(B.counter, static_cast<unsigned long long>(blockIdx.x) * blockDim.x + tid, BP.total,
              static_cast<unsigned long long>(gridDim.x) * blockDim.x);
    Photon p;
    p.media = 0;
    p.lastvox = -1;
    bool active = false, done = false;
    int sim = 0, tally_sim = -1;
    etally[tid] = 0.0;  // per-lane FP64 tallies of the current simulation, in shared memory
    etally[blockDim.x + tid] = 0.0;
    Counters c;

    for (unsigned iter = 0;; iter++) {
        if (!active && !done) {
            unsigned long long g;
            if (!feed.take(B.counter, &g, BP.total)) {
                done = true;
            } else {
                int lo = 0, hi = BP.nsim - 1;  // largest s with begin[s] <= g
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (begin[mid] <= g) lo = mid;
                    else hi = mid - 1;
                }
                sim = lo;
                if (sim != tally_sim) {
                    if (tally_sim >= 0 && (etally[blockDim.x + tid] != 0.0 || etally[tid] != 0.0)) {
                        atomicAdd(BP.tallies + 2 * tally_sim, etally[tid]);
                        atomicAdd(BP.tallies + 2 * tally_sim + 1, etally[blockDim.x + tid]);
                    }
                    tally_sim = sim;
                    etally[blockDim.x + tid] = 0.0;
                    etally[tid] = 0.0;
                }
                const SimDesc& S = sd[sim];
                rare_count(kRareLaunch);
                const GlobalLabels lab = global_labels(B, S.label_off, S.dimxyz, BP.total_media - S.media_base);
                active = start_photon<false>(S, lab, p, S.photon_offset + (g - begin[sim]));
                if (SAVEDET && active)
                    for (int q = 0; q < S.ppathlen; q++) ppath[q * blockDim.x + tid] = 0.f;
            }
        }
        // warp-uniform exits, tested every 16 iterations (a finished lane idles for at most 15 more)
        if ((iter & 15u) == 0u) {
            if (__all_sync(kFull, done)) break;
            if (out_of_budget(B, iter, lane)) break;
        }

        bool term = false;
        if (AGG) {  // deposits after the divergent part, aggregated per warp
            long long dep_idx = -1;
            float dep_val = 0.f;
            Event ev;
            ev.term = false;
            if (active) {
                const SimDesc& S = sd[sim];
                const GlobalLabels lab = global_labels(B, S.label_off, S.dimxyz, BP.total_media - S.media_base);
                advance<false, REFLECT, false>(S, lab, sm + S.media_base, p, ev, c);
                if (SAVEDET && ev.crossed && ev.left_mid - 1u < static_cast<unsigned>(S.ppathlen))
                    ppath[(ev.left_mid - 1) * blockDim.x + tid] += ev.seg;  // L286-288
                const bool dep = ev.crossed && S.issavevol && ev.gate >= 0;
                dep_idx = dep ? static_cast<long long>(S.out_off) + ev.left_vox +
                                    static_cast<long long>(ev.gate) * static_cast<long long>(S.dimxyz)
                              : -1;
                dep_val = dep ? ev.dep_val : 0.f;
            }
            const unsigned hm = __ballot_sync(kFull, dep_idx >= 0);
            if (__popc(hm) > 1) {
                const unsigned grp = __match_any_sync(kFull, dep_idx >= 0 ? static_cast<unsigned long long>(dep_idx) : ~0ULL);
                aggbuf[tid] = dep_val;
                __syncwarp();
                if (dep_idx >= 0 && lane == __ffs(grp) - 1u) {
                    float s = 0.f;
                    const unsigned base = tid & ~31u;
                    for (unsigned gm = grp; gm; gm &= gm - 1) s += aggbuf[base + __ffs(gm) - 1];
                    deposit_add64(B, dep_idx, s);
                }
                __syncwarp();
            } else if (dep_idx >= 0) {
                deposit_add64(B, dep_idx, dep_val);
            }
            term = ev.term;
        } else if (active) {  // plain atomics where the crossing is handled
            const SimDesc& S = sd[sim];
            const GlobalLabels lab = global_labels(B, S.label_off, S.dimxyz, BP.total_media - S.media_base);
            term = photon_step<false, REFLECT, false>(
                S, lab, sm + S.media_base, p, c,
                [&](unsigned mid, const Medium& m) {
                    record_crossing<false, SAVEDET>(S, p, mid, m, ppath + tid, &B.stats->error, [&](int vox, int gate, float v) {
                        deposit_add64(B, static_cast<long long>(S.out_off) + vox + static_cast<long long>(gate) * S.dimxyz,
                                      v);
                    });
                },
                [](unsigned) {});
        }
        if (term) {
            count_stopped(p);
            if (!AGG) c.steps += p.nsteps;  // photon_step does not count steps one by one
            if (SAVEDET) {
                const SimDesc& S = sd[sim];
                if ((p.media & UMCX_LABEL_DET) && p.ly <= S.tend)  // L276-278, L429-435
                    for (int d = 0; d < S.detnum; d++) {
                        if (!det_hit(sdet[S.det_base + d], p)) continue;
                        const unsigned long long slot = atomicAdd(BP.detected + sim, 1ULL);
                        if (slot < S.maxdetphotons) write_detp(S, B, p, ppath + tid, blockDim.x, d, slot, S.detp_off);
                    }
            }
            if ((p.media & UMCX_LABEL_MASK) != 0u) {
                etally[blockDim.x + tid] += p.launchw;
                etally[tid] += p.pw;
            }
            active = false;
        }
    }
    if (tally_sim >= 0 && (etally[blockDim.x + tid] != 0.0 || etally[tid] != 0.0)) {
        atomicAdd(BP.tallies + 2 * tally_sim, etally[tid]);
        atomicAdd(BP.tallies + 2 * tally_sim + 1, etally[blockDim.x + tid]);
    }
    flush_tallies(B, lane, 0.0, 0.0, c);
    rare_flush(B);
}

// detector readings and their per-label derivatives from the extended records (FP64 accumulation):
//   R[d][t] += w,  dR/dmua_k[d][t] += -w L_k,  dR/dmus_k[d][t] += w (n_k / mus_k - L_k)
__global__ void k_adjoint_reduce(const KParams P, const DetRecord* __restrict__ rec, const float* __restrict__ ext,
                                 unsigned long long n, const Medium* __restrict__ media, double* __restrict__ read,
                                 double* __restrict__ gmua, double* __restrict__ gmus);

// rand01 known-answer dump (MCX_rand, L187-215)
__global__ void k_rng_dump(unsigned s0, unsigned s1, unsigned s2, unsigned s3, unsigned long long offset,
                           unsigned nphoton, unsigned ndraw, float* out);

}  // namespace umcx_dev
