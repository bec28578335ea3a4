/*
 * umcx_oracle.c - CPU oracle for the umcx photon-transport hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load this
 * file's library, and only to compute expected results; the product (umcx_gb300/) never calls it and has no CPU fallback.
 *
 * A plain-C restatement of the reference's photon loop (fangq/umcx, src/umcx.cpp), written to follow the
 * reference's floating-point expression order so that, single-threaded on x86-64 with -ffp-contract=off, its
 * output volume and detected-photon rows equal the reference binary's bit for bit (pinned against the
 * reference's own outputs by tests/test_oracle_pin.py).  The RNG and seed derivation are reproduced exactly on
 * every platform.
 *
 * Differences in representation only (semantics unchanged): labels are uint8 with bit 7 as the detector flag
 * (the reference uses int32 with the sign bit, L35-36); the photon index range is [photon_offset,
 * photon_offset + nphoton) instead of [0, nphoton) so that ranges can be split for batch statistics.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/umcx_gpu.h"

#define ORC_ONE_OVER_C0 3.335640951981520e-12f /* L29 */
#define ORC_PI 3.1415926535897932385f          /* L30 */

typedef struct { float x, y, z, w; } f4;

/* ---- xorshift128+ (MCX_rand, L187-215) ---- */
typedef struct { uint64_t t0, t1; } orc_rng;

static void orc_reseed(orc_rng* r, uint32_t s0, uint32_t s1, uint32_t s2, uint32_t s3) { /* L193-196 */
    r->t0 = ((uint64_t)s0 << 32) | s1;
    r->t1 = ((uint64_t)s2 << 32) | s3;
}

static float orc_rand01(orc_rng* r) { /* L197-211 */
    uint64_t a = r->t0;
    const uint64_t b = r->t1;
    r->t0 = b;
    a ^= a << 23;
    r->t1 = a ^ b ^ (a >> 18) ^ (b >> 5);
    uint32_t lo = (uint32_t)(r->t1 + b);
    union { uint32_t u; float f; } c;
    c.u = 0x3F800000u | (lo >> 9);
    return c.f - 1.0f;
}

static float orc_scatlen(orc_rng* r) { return -logf(orc_rand01(r) + FLT_EPSILON); } /* L212-214 */

/* ---- photon state (MCX_photon members, L218-220) ---- */
typedef struct {
    f4 pos;   /* x, y, z, weight */
    f4 vec;   /* direction, scatter count */
    f4 rvec;  /* 1/direction, scratch */
    f4 len;   /* remaining scattering length, time, path since last deposit, weight at last deposit */
    int16_t ix, iy, iz, flip;
    int lastvox, media;
    unsigned nsteps, zsteps;  /* step count and consecutive zero-length steps (guards, see orc_sprint) */
} orc_photon;

typedef struct {
    const umcx_sim* s;
    const uint8_t* labels;
    const f4* media;
    const f4* det;
    float* fluence;
    float* detp;
    uint32_t* depcount;
    uint64_t* detected;
    uint32_t dimyz, dimxyz;
    int cols, ppathlen;
    float* trace; int trace_max; int* trace_n;   /* optional per-event trace of one photon */
} orc_ctx;

static int orc_index(const orc_ctx* c, int16_t ix, int16_t iy, int16_t iz) { /* MCX_volume::index, L128-130 */
    const umcx_sim* s = c->s;
    return !(ix < 0 || iy < 0 || iz < 0 || ix >= (int16_t)s->dim[0] || iy >= (int16_t)s->dim[1] ||
             iz >= (int16_t)s->dim[2])
               ? (int)((uint64_t)ix * c->dimyz + (uint64_t)iy * s->dim[2] + (uint64_t)iz)
               : -1;
}

static void orc_trace(const orc_ctx* c, int kind, const orc_photon* p) {
    if (!c->trace || *c->trace_n >= c->trace_max) return;
    float* t = c->trace + 8 * (*c->trace_n)++;
    t[0] = (float)kind; t[1] = p->pos.x; t[2] = p->pos.y; t[3] = p->pos.z;
    t[4] = p->pos.w; t[5] = p->vec.x; t[6] = p->vec.y; t[7] = p->vec.z;
}

static void orc_rotate(orc_photon* p, float stheta, float ctheta, float sphi, float cphi) { /* L418-428 */
    f4 v = p->vec;
    if (v.z > -1.f + FLT_EPSILON && v.z < 1.f - FLT_EPSILON) {
        float tmp0 = 1.f - v.z * v.z, tmp1 = stheta / sqrtf(tmp0);
        p->vec.x = tmp1 * (v.x * v.z * cphi - v.y * sphi) + v.x * ctheta;
        p->vec.y = tmp1 * (v.y * v.z * cphi + v.x * sphi) + v.y * ctheta;
        p->vec.z = -tmp1 * tmp0 * cphi + v.z * ctheta;
    } else {
        p->vec.x = stheta * cphi;
        p->vec.y = stheta * sphi;
        p->vec.z = (v.z > 0.f) ? ctheta : -ctheta;
    }
    float norm = 1.f / sqrtf(p->vec.x * p->vec.x + p->vec.y * p->vec.y + p->vec.z * p->vec.z);
    p->vec.x *= norm; p->vec.y *= norm; p->vec.z *= norm;
}

static float orc_launch(const orc_ctx* c, orc_photon* p, orc_rng* r) { /* MCX_photon::launch, L225-259 */
    const umcx_sim* s = c->s;
    const f4 v0 = {s->srcdir[0], s->srcdir[1], s->srcdir[2], 0.f};
    p->pos.x = s->srcpos[0]; p->pos.y = s->srcpos[1]; p->pos.z = s->srcpos[2]; p->pos.w = 1.f;
    p->vec = v0;
    const float* p1 = s->srcparam1;
    const float* p2 = s->srcparam2;
    if (s->srctype == UMCX_SRC_ISOTROPIC || s->srctype == UMCX_SRC_CONE) { /* L228-234 */
        float phi = (ORC_PI * 2.f) * orc_rand01(r);
        float sphi = sinf(phi), cphi = cosf(phi);
        float theta;
        if (s->srctype == UMCX_SRC_ISOTROPIC) {
            theta = acosf(2.f * orc_rand01(r) - 1.f);
        } else {
            float c0 = cosf(p1[0]);
            theta = acosf(orc_rand01(r) * (1.0f - c0) + c0);
        }
        orc_rotate(p, sinf(theta), cosf(theta), sphi, cphi);
    } else if (s->srctype == UMCX_SRC_DISK) { /* L235-247 */
        float phi = (ORC_PI * 2.f) * orc_rand01(r);
        float sphi = sinf(phi), cphi = cosf(phi);
        float rad = sqrtf(orc_rand01(r) * fabsf(p1[0] * p1[0] - p1[1] * p1[1]) + p1[1] * p1[1]);
        if (p->vec.z > -1.f + FLT_EPSILON && p->vec.z < 1.f - FLT_EPSILON) {
            float l = 1.f - p->vec.z * p->vec.z;
            float q = rad / sqrtf(l);
            f4 np;
            np.x = p->pos.x + q * (p->vec.x * p->vec.z * cphi - p->vec.y * sphi);
            np.y = p->pos.y + q * (p->vec.y * p->vec.z * cphi + p->vec.x * sphi);
            np.z = p->pos.z - q * l * cphi;
            np.w = p->pos.w;
            p->pos = np;
        } else {
            p->pos.x += rad * cphi;
            p->pos.y += rad * sphi;
        }
    } else if (s->srctype == UMCX_SRC_PLANAR || s->srctype == UMCX_SRC_FOURIER) { /* L248-253 */
        float a = orc_rand01(r);
        float b = orc_rand01(r);
        f4 np;
        np.x = p->pos.x + a * p1[0] + b * p2[0];
        np.y = p->pos.y + a * p1[1] + b * p2[1];
        np.z = p->pos.z + a * p1[2] + b * p2[2];
        np.w = p->pos.w;
        p->pos = np;
        p->pos.w *= (s->srctype == UMCX_SRC_FOURIER)
                        ? (cosf((floorf(p1[3]) * a + floorf(p2[3]) * b + p1[3] - floorf(p1[3])) * ORC_PI * 2.f) *
                               (1.f - p2[3] + floorf(p2[3])) +
                           1.f) *
                              0.5f
                        : 1.f;
    }
    /* L255-257: the inverse direction is taken from the ORIGINAL source direction, also for rotated
     * isotropic/cone launches */
    p->rvec.x = 1.f / v0.x; p->rvec.y = 1.f / v0.y; p->rvec.z = 1.f / v0.z; p->rvec.w = 0.f;
    p->len.x = NAN; p->len.y = 0.f; p->len.z = 0.f; p->len.w = p->pos.w;
    p->ix = (int16_t)p->pos.x; p->iy = (int16_t)p->pos.y; p->iz = (int16_t)p->pos.z; p->flip = -1;
    return p->pos.w;
}

static float orc_skip(const orc_ctx* c, orc_photon* p) { /* MCX_photon::skip, L339-358 */
    const umcx_sim* s = c->s;
    float ax = -p->pos.x * p->rvec.x, ay = -p->pos.y * p->rvec.y, az = -p->pos.z * p->rvec.z;
    float bx = ((float)s->dim[0] - p->pos.x) * p->rvec.x;
    float by = ((float)s->dim[1] - p->pos.y) * p->rvec.y;
    float bz = ((float)s->dim[2] - p->pos.z) * p->rvec.z;
    float tmin = fmaxf(fmaxf(fminf(ax, bx), fminf(ay, by)), fminf(az, bz));
    float tmax = fminf(fminf(fmaxf(ax, bx), fmaxf(ay, by)), fmaxf(az, bz));
    if (tmax < 0.f || tmin > tmax) return -1.f;
    p->pos.x = p->pos.x + tmin * p->vec.x;
    p->pos.y = p->pos.y + tmin * p->vec.y;
    p->pos.z = p->pos.z + tmin * p->vec.z;
    p->pos.w = 1.f; /* the launch weight is reset to 1 here (L353) */
    p->len.x = NAN; p->len.y = 0.f; p->len.z = 0.f; p->len.w = p->pos.w;
    p->ix = (int16_t)p->pos.x; p->iy = (int16_t)p->pos.y; p->iz = (int16_t)p->pos.z; p->flip = -1;
    p->lastvox = orc_index(c, p->ix, p->iy, p->iz);
    return tmin;
}

static int orc_step(const orc_ctx* c, orc_photon* p, const f4 prop) { /* MCX_photon::step, L315-338 */
    float hx = fabsf(((float)(p->ix + (p->vec.x > 0.f)) - p->pos.x) * p->rvec.x);
    float hy = fabsf(((float)(p->iy + (p->vec.y > 0.f)) - p->pos.y) * p->rvec.y);
    float hz = fabsf(((float)(p->iz + (p->vec.z > 0.f)) - p->pos.z) * p->rvec.z);
    float dist = fminf(fminf(hx, hy), hz);
    p->flip = (dist == hx ? 0 : (dist == hy ? 1 : 2));
    float used = fminf(dist * prop.y, p->len.x);
    int cross = (used != p->len.x);
    dist = (prop.y == 0.f) ? dist : (used / prop.y);
    p->rvec.w = dist;
    p->pos.x = p->pos.x + dist * p->vec.x;
    p->pos.y = p->pos.y + dist * p->vec.y;
    p->pos.z = p->pos.z + dist * p->vec.z;
    p->pos.w = p->pos.w * expf(-prop.x * dist);
    p->len.x -= used;
    p->len.y += dist * prop.w * ORC_ONE_OVER_C0;
    p->len.z += dist;
    if (cross) {
        if (p->flip == 0) p->ix += (p->vec.x > 0.f ? 1 : -1);
        else if (p->flip == 1) p->iy += (p->vec.y > 0.f ? 1 : -1);
        else p->iz += (p->vec.z > 0.f ? 1 : -1);
        return orc_index(c, p->ix, p->iy, p->iz);
    }
    return p->lastvox;
}

static void orc_save(const orc_ctx* c, orc_photon* p, int gate, float mua) { /* MCX_photon::save, L359-363 */
    const umcx_sim* s = c->s;
    float v = s->outputtype == UMCX_OUT_ENERGY ? (p->len.w - p->pos.w)
                                               : (mua < FLT_EPSILON ? (p->len.w * p->len.z) : (p->len.w - p->pos.w) / mua);
    if (gate >= 0) { /* the reference writes out of bounds for gate < 0 (time before tstart); skipped here */
        uint64_t idx = (uint64_t)p->lastvox + (uint64_t)gate * c->dimxyz;
#pragma omp atomic
        c->fluence[idx] += v;
        if (c->depcount) {
#pragma omp atomic
            c->depcount[idx] += 1u;
        }
    }
    p->len.w = p->pos.w;
    p->len.z = 0.f;
}

static void orc_scatter(orc_photon* p, const f4 prop, orc_rng* r) { /* MCX_photon::scatter, L364-380 */
    p->len.x = orc_scatlen(r);
    float tmp0 = (2.f * ORC_PI) * orc_rand01(r);
    float sphi = sinf(tmp0), cphi = cosf(tmp0);
    float stheta, ctheta, th;
    if (fabsf(prop.z) > FLT_EPSILON) {
        tmp0 = (1.f - prop.z * prop.z) / (1.f - prop.z + 2.f * prop.z * orc_rand01(r));
        tmp0 = (1.f + prop.z * prop.z - tmp0 * tmp0) / (2.f * prop.z);
        th = acosf(fmaxf(-1.f, fminf(1.f, tmp0)));
    } else {
        th = acosf(2.f * orc_rand01(r) - 1.f);
    }
    stheta = sinf(th); ctheta = cosf(th);
    orc_rotate(p, stheta, ctheta, sphi, cphi);
    p->rvec.x = 1.f / p->vec.x; p->rvec.y = 1.f / p->vec.y; p->rvec.z = 1.f / p->vec.z; p->rvec.w = cphi;
    p->vec.w++;
}

static float orc_reflectcoeff(const orc_photon* p, float n1, float n2) { /* L381-395 */
    float Icos = fabsf((p->flip == 0) ? p->vec.x : (p->flip == 1 ? p->vec.y : p->vec.z));
    float tmp0 = n1 * n1, tmp1 = n2 * n2;
    float tmp2 = 1.f - tmp0 / tmp1 * (1.f - Icos * Icos);
    if (tmp2 > 0.f) {
        float Re = tmp0 * Icos * Icos + tmp1 * tmp2;
        tmp2 = sqrtf(tmp2);
        float Im = 2.f * n1 * n2 * Icos * tmp2;
        float Rtotal = (Re - Im) / (Re + Im);
        Re = tmp1 * Icos * Icos + tmp0 * tmp2 * tmp2;
        return (Rtotal + (Re - Im) / (Re + Im)) * 0.5f;
    }
    return 1.f;
}

static float orc_sign(float v) { return (float)((v > 0.f) - (v < 0.f)); }

/* returns 1 when transmitted; on reflection updates newvox/newmedia to the current voxel (L405-417) */
static int orc_reflect(orc_photon* p, float n1, float n2, orc_rng* r, int* newvox, int* newmedia) {
    float Rtotal = orc_reflectcoeff(p, n1, n2);
    if (Rtotal < 1.f && orc_rand01(r) > Rtotal) { /* transmit, L396-404 */
        float k = n1 / n2;
        p->vec.x *= k; p->vec.y *= k; p->vec.z *= k;
        float* comp = p->flip == 0 ? &p->vec.x : (p->flip == 1 ? &p->vec.y : &p->vec.z);
        float t = p->vec.x * p->vec.x + p->vec.y * p->vec.y + p->vec.z * p->vec.z - (*comp) * (*comp);
        *comp = (t < 1.f) ? sqrtf(1.f - t) * orc_sign(*comp) : 0.f;
        float norm = 1.f / sqrtf(p->vec.x * p->vec.x + p->vec.y * p->vec.y + p->vec.z * p->vec.z);
        p->vec.x *= norm; p->vec.y *= norm; p->vec.z *= norm;
        /* the inverse direction is not refreshed after refraction (as in the reference) */
        return 1;
    }
    /* REFLECT_PHOTON, L31 */
    if (p->flip == 0) {
        p->vec.x = -p->vec.x; p->rvec.x = -p->rvec.x;
        p->pos.x = nextafterf((float)(int)(p->pos.x + 0.5f), orc_sign(p->vec.x)); p->ix = (int16_t)p->pos.x;
    } else if (p->flip == 1) {
        p->vec.y = -p->vec.y; p->rvec.y = -p->rvec.y;
        p->pos.y = nextafterf((float)(int)(p->pos.y + 0.5f), orc_sign(p->vec.y)); p->iy = (int16_t)p->pos.y;
    } else {
        p->vec.z = -p->vec.z; p->rvec.z = -p->rvec.z;
        p->pos.z = nextafterf((float)(int)(p->pos.z + 0.5f), orc_sign(p->vec.z)); p->iz = (int16_t)p->pos.z;
    }
    *newvox = p->lastvox;
    *newmedia = p->media;
    return 0;
}

typedef struct { uint64_t steps, crossings, scatters, reflections; } orc_events;

/* MCX_photon::sprint, L281-314: returns 1 when the photon terminates */
static int orc_sprint(const orc_ctx* c, orc_photon* p, orc_rng* r, float* ppath, orc_events* ev) {
    const umcx_sim* s = c->s;
    while (p->len.x > 0.f) {
        int newvox = orc_step(c, p, c->media[p->media & UMCX_LABEL_MASK]);
        ev->steps++;
        /* Guards absent from the reference (which would loop forever): a photon stops after 2^24 steps, or after
         * 255 consecutive zero-length steps (a zero direction component at a grid face can bounce between a
         * zero-length crossing and a reflection in place).  Terminating photons never reach either limit, so
         * outputs are unchanged; the CUDA kernels apply the same rule. */
        p->zsteps = (p->rvec.w == 0.f) ? p->zsteps + 1 : 0;
        if (++p->nsteps > (1u << 24) || p->zsteps >= 255) return 1;
        if (newvox != p->lastvox) {
            ev->crossings++;
            if (s->issavedet && (s->savedetflag & UMCX_DET_PPATH) && ((p->media & UMCX_LABEL_MASK) > 0)) {
                ppath[(p->media & UMCX_LABEL_MASK) - 1] += p->len.z;
            }
            if (s->issavevol) {
                int gate = (int)fminf((float)(s->dim[3] - 1), (float)(int)(floorf((p->len.y - s->tstart) * s->rtstep)));
                orc_save(c, p, gate, c->media[p->media & UMCX_LABEL_MASK].x);
            }
            orc_trace(c, 1, p);
            if (p->len.y > s->tend) return 1;
            int newmedia = (newvox >= 0) ? c->labels[newvox] : 0;
            if (s->isreflect && c->media[p->media & UMCX_LABEL_MASK].w != c->media[newmedia & UMCX_LABEL_MASK].w) {
                ev->reflections++;
                if (orc_reflect(p, c->media[p->media & UMCX_LABEL_MASK].w, c->media[newmedia & UMCX_LABEL_MASK].w, r,
                                &newvox, &newmedia) &&
                    (newvox < 0 || (newmedia & UMCX_LABEL_MASK) == 0)) {
                    return 1;
                }
            } else if (newvox < 0 || ((newmedia & UMCX_LABEL_MASK) == 0 && (p->media & UMCX_LABEL_MASK) != 0)) {
                return 1;
            }
            p->lastvox = newvox;
            p->media = newmedia;
        }
    }
    return 0;
}

/* MCX_detect::addphoton (L164-176) and MCX_photon::savedetector (L429-435) */
static void orc_savedetector(const orc_ctx* c, const orc_photon* p, const float* ppath) {
    const umcx_sim* s = c->s;
    for (int i = 0; i < s->detnum; i++) {
        const f4 d = c->det[i];
        if ((d.x - p->pos.x) * (d.x - p->pos.x) + (d.y - p->pos.y) * (d.y - p->pos.y) +
                (d.z - p->pos.z) * (d.z - p->pos.z) <
            d.w * d.w) {
            uint64_t slot;
#pragma omp atomic capture
            slot = (*c->detected)++;
            if (slot < s->maxdetphotons && c->detp) {
                float* rec = c->detp + slot * (uint64_t)c->cols;
                int k = 0;
                if (s->savedetflag & UMCX_DET_ID) rec[k++] = (float)(i + 1);
                if (s->savedetflag & UMCX_DET_PPATH)
                    for (int m = 0; m < c->ppathlen; m++) rec[k++] = ppath[m];
                if (s->savedetflag & UMCX_DET_EXITPOS) { rec[k++] = p->pos.x; rec[k++] = p->pos.y; rec[k++] = p->pos.z; }
                if (s->savedetflag & UMCX_DET_EXITDIR) { rec[k++] = p->vec.x; rec[k++] = p->vec.y; rec[k++] = p->vec.z; }
            }
        }
    }
}

int oracle_detp_columns(const umcx_sim* s) { /* L157 */
    return (s->savedetflag & UMCX_DET_ID) + ((s->savedetflag & UMCX_DET_PPATH) > 0) * s->mediumnum +
           (((s->savedetflag & UMCX_DET_EXITPOS) > 0) + ((s->savedetflag & UMCX_DET_EXITDIR) > 0)) * 3;
}

/* the four session seeds: srand(seed) + 4 x rand() of the C library (L724-727), via the reentrant API so the
 * caller's global rand() state is untouched */
int oracle_seeds(int32_t rngseed, uint32_t out[4]) {
    struct random_data rd;
    char state[128];
    memset(&rd, 0, sizeof(rd));
    memset(state, 0, sizeof(state));
    if (initstate_r((unsigned)rngseed, state, sizeof(state), &rd) != 0) return 1;
    for (int i = 0; i < 4; i++) {
        int32_t v;
        random_r(&rd, &v);
        out[i] = (uint32_t)v;
    }
    return 0;
}

void oracle_rng_dump(const uint32_t seeds[4], uint64_t photon, int ndraw, float* out) {
    orc_rng r;
    orc_reseed(&r, seeds[0] ^ (uint32_t)photon, seeds[1] | (uint32_t)photon, seeds[2] ^ (uint32_t)photon,
               seeds[3] | (uint32_t)photon);
    for (int i = 0; i < ndraw; i++) out[i] = orc_rand01(&r);
}

/* Runs one photon (L761-770 body); returns 1 when the photon is counted in the energy totals. */
static int orc_photon_run(const orc_ctx* c, uint64_t i, orc_events* ev, float* launchw, float* finalw,
                          float* ppath_out) {
    const umcx_sim* s = c->s;
    float ppath[UMCX_MAX_MEDIA];
    orc_rng r;
    orc_photon p;
    memset(&p, 0, sizeof(p));
    memset(ppath, 0, sizeof(float) * (size_t)(s->mediumnum > 0 ? s->mediumnum : 1));
    orc_reseed(&r, s->seeds[0] ^ (uint32_t)i, s->seeds[1] | (uint32_t)i, s->seeds[2] ^ (uint32_t)i,
               s->seeds[3] | (uint32_t)i);
    *launchw = orc_launch(c, &p, &r);
    orc_trace(c, 0, &p);
    /* MCX_photon::run, L261-279 */
    p.lastvox = orc_index(c, p.ix, p.iy, p.iz);
    if (p.lastvox < 0 && (orc_skip(c, &p) < 0.f || p.lastvox < 0)) {
        p.media = 0;
        *finalw = p.pos.w;
        return 0;
    }
    p.media = c->labels[p.lastvox];
    p.len.x = orc_scatlen(&r);
    while (orc_sprint(c, &p, &r, ppath, ev) == 0) {
        orc_scatter(&p, c->media[p.media & UMCX_LABEL_MASK], &r);
        ev->scatters++;
        orc_trace(c, 2, &p);
    }
    if (s->issavedet && (p.media & UMCX_LABEL_DET) && p.len.y <= s->tend) orc_savedetector(c, &p, ppath);
    *finalw = p.pos.w;
    if (ppath_out) memcpy(ppath_out, ppath, sizeof(float) * (size_t)s->mediumnum);
    return (p.media & UMCX_LABEL_MASK) != 0;
}

static int orc_setup(orc_ctx* c, const umcx_sim* s, const uint8_t* labels, const float* media, const float* detpos,
                     float* fluence, float* detp, uint32_t* depcount, uint64_t* detected) {
    memset(c, 0, sizeof(*c));
    if (s->mediumnum < 1 || s->mediumnum > UMCX_MAX_MEDIA || s->dim[3] < 1) return 1;
    c->s = s;
    c->labels = labels;
    c->media = (const f4*)media;
    c->det = (const f4*)detpos;
    c->fluence = fluence;
    c->detp = detp;
    c->depcount = depcount;
    c->detected = detected;
    c->dimyz = s->dim[1] * s->dim[2];
    c->dimxyz = c->dimyz * s->dim[0];
    c->cols = oracle_detp_columns(s);
    c->ppathlen = (s->issavedet && (s->savedetflag & UMCX_DET_PPATH)) ? s->mediumnum : 0;
    return 0;
}

/*
 * MCX_kernel (L722-781) over photons [photon_offset, photon_offset + nphoton).  fluence (maxgate*nx*ny*nz) is
 * accumulated into (not cleared); detp receives up to maxdetphotons rows; depcount (optional) counts deposits
 * per output element.  nthreads <= 0 uses the OpenMP default.
 */
int oracle_forward(const umcx_sim* s, const uint8_t* labels, const float* media, const float* detpos, float* fluence,
                   float* detp, uint32_t* depcount, umcx_result* res, int nthreads) {
    orc_ctx c;
    uint64_t detected = 0;
    if (orc_setup(&c, s, labels, media, detpos, fluence, detp, depcount, &detected)) return UMCX_ERR_INPUT;
    double esc = 0.0, tot = 0.0;
    uint64_t steps = 0, crossings = 0, scatters = 0, reflections = 0;
    const int64_t n = (int64_t)s->nphoton;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : esc, tot, steps, crossings, scatters, reflections)
    for (int64_t k = 0; k < n; k++) {
        orc_events ev = {0, 0, 0, 0};
        float lw, fw;
        if (orc_photon_run(&c, s->photon_offset + (uint64_t)k, &ev, &lw, &fw, NULL)) {
            tot += lw;
            esc += fw;
        }
        steps += ev.steps; crossings += ev.crossings; scatters += ev.scatters; reflections += ev.reflections;
    }
    if (res) {
        memset(res, 0, sizeof(*res));
        res->energy_escape = esc;
        res->energy_total = tot;
        res->detected = detected;
        res->saved = detected < s->maxdetphotons ? detected : s->maxdetphotons;
        res->launched = s->nphoton;
        res->steps = steps; res->crossings = crossings; res->scatters = scatters; res->reflections = reflections;
    }
    return UMCX_OK;
}

/*
 * Event trace of ONE photon (launch = kind 0, voxel crossing = 1, scatter = 2), rows of 8 floats
 * {kind, x, y, z, weight, vx, vy, vz}.  Returns the number of rows written (at most maxrows).  The fluence
 * side effects go to a caller scratch buffer.
 */
int oracle_trace_photon(const umcx_sim* s, const uint8_t* labels, const float* media, const float* detpos,
                        uint64_t photon, float* scratch_fluence, float* rows, int maxrows) {
    orc_ctx c;
    uint64_t detected = 0;
    int n = 0;
    if (orc_setup(&c, s, labels, media, detpos, scratch_fluence, NULL, NULL, &detected)) return -1;
    c.trace = rows; c.trace_max = maxrows; c.trace_n = &n;
    orc_events ev = {0, 0, 0, 0};
    float lw, fw;
    orc_photon_run(&c, photon, &ev, &lw, &fw, NULL);
    return n;
}
