/*
 * umcx_gpu.h - C ABI of the GB300 photon-transport library (libumcx_gb300.so).
 *
 * Plain C types only: pointers, sizes, PODs.  Every entry point returns an int status (UMCX_OK = 0) and
 * never lets a C++ exception cross the boundary; the message of the last failure on a context is returned by
 * umcx_last_error().
 *
 * Reference interfaces replaced (fangq/umcx, src/umcx.cpp):
 *   MCX_run_cmd / MCX_run_json            src/umcx.cpp:850-856  (same symbols, same argv / JSON semantics)
 *   MCX_kernel<isreflect,issavedet>()     src/umcx.cpp:722-781  (-> umcx_gpu_forward*)
 *   MCX_param                              src/umcx.cpp:95-99    (-> umcx_sim)
 *   MCX_medium                             src/umcx.cpp:89-93    (-> float[4] {mua, mus, g, n} per label)
 *   MCX_volume<int> labels + DET_MASK      src/umcx.cpp:102-146, 35-36 (-> uint8 labels, bit 7 = detector voxel)
 *   MCX_volume<float> output               src/umcx.cpp:102-146  (-> float fluence [gate][x][y][z])
 *   MCX_detect                             src/umcx.cpp:149-185  (-> float detp [saved][cols])
 *   seeds from std::srand/std::rand        src/umcx.cpp:724-727  (-> umcx_seeds_from_rngseed)
 * Entry points with no reference counterpart (the reference has no adjoint, replay or batching) say so.
 */
#ifndef UMCX_GPU_H
#define UMCX_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define UMCX_ABI_VERSION 4

/* status codes */
enum {
    UMCX_OK = 0,
    UMCX_ERR_INPUT = 1,   /* invalid argument or configuration (reference: std::runtime_error, L514/L520/L570/L667) */
    UMCX_ERR_CUDA = 2,    /* a CUDA runtime call failed */
    UMCX_ERR_TIMEOUT = 3, /* the device-side step cap or deadline was hit; partial results are returned */
    UMCX_ERR_NODEV = 4    /* no usable CUDA device */
};

/* output types, same order as the reference's "xfe" (L57-58) */
enum { UMCX_OUT_FLUENCE_RATE = 0, UMCX_OUT_FLUENCE = 1, UMCX_OUT_ENERGY = 2 };
/* source types, same order as the reference's list (L59-60) */
enum { UMCX_SRC_PENCIL = 0, UMCX_SRC_ISOTROPIC = 1, UMCX_SRC_CONE = 2, UMCX_SRC_DISK = 3, UMCX_SRC_PLANAR = 4,
       UMCX_SRC_FOURIER = 5 };
/* detected-photon record flags (L65) */
enum { UMCX_DET_ID = 1, UMCX_DET_PPATH = 4, UMCX_DET_EXITPOS = 16, UMCX_DET_EXITDIR = 32 };

/* bit 7 of a label byte marks a detector voxel (the reference uses the sign bit of an int32 label, L35-36, L622) */
#define UMCX_LABEL_DET 0x80u
#define UMCX_LABEL_MASK 0x7Fu
/* largest medium count: labels are 7-bit */
#define UMCX_MAX_MEDIA 128
/* largest detector count handled by the device kernels */
#define UMCX_MAX_DET 64
/* largest time-gate count */
#define UMCX_MAX_GATES 65535

/* umcx_sim.flags bits */
#define UMCX_SIM_STRICT_MATH 0x1u /* evaluate every expression like the reference (IEEE division, expf/logf/
                                     sinf/cosf/acosf, no FMA contraction) instead of the fast hardware forms */
#define UMCX_SIM_FP32_ACCUM 0x2u /* accumulate the output volume with FP32 atomics directly in `fluence`, like the
                                    reference (MCX_volume::add, L134-137).  Default: FP64 accumulation in a
                                    library-owned volume, rounded to FP32 once at the end; FP32 accumulation loses
                                    small deposits in heavily hit voxels (2e-5 of the energy at 1e6 photons). */
#define UMCX_SIM_FLAGS_ALL 0x3u

/*
 * One simulation.  Field meanings follow MCX_param (L95-99) as filled at L787-796, plus the inputs MCX_kernel
 * reads itself (photon count L726, seeds L725-727, source L728-729).  mua and mus in the media table are in
 * per-voxel units, i.e. already multiplied by unitinmm as at L804.
 */
typedef struct umcx_sim {
    uint32_t dim[4];          /* nx, ny, nz, maxgate (L789) */
    uint64_t nphoton;         /* photons to launch */
    uint64_t photon_offset;   /* index of the first photon; photon i is reseeded from (seeds, i) (L761) */
    float tstart, tend, rtstep, unitinmm;
    int32_t isreflect;        /* DoMismatch */
    int32_t issavevol;        /* DoSaveVolume */
    int32_t issavedet;        /* DoPartialPath */
    int32_t savedetflag;      /* SaveDetFlag, sum of UMCX_DET_* */
    int32_t mediumnum;        /* media count including label 0 */
    int32_t outputtype;       /* UMCX_OUT_* */
    int32_t detnum;           /* detectors */
    int32_t srctype;          /* UMCX_SRC_* */
    uint32_t maxdetphotons;   /* MaxDetPhoton */
    uint32_t flags;           /* UMCX_SIM_* bits (0 = production fast path) */
    uint32_t seeds[4];        /* the four 32-bit session seeds */
    float srcpos[4];          /* source position (w = initial weight, 1) */
    float srcdir[4];          /* source direction */
    float srcparam1[4];
    float srcparam2[4];
} umcx_sim;

/* Per-call results (not normalised; the host applies the normaliser of L820). */
typedef struct umcx_result {
    double energy_escape;     /* L768-769 */
    double energy_total;      /* L766-767 */
    uint64_t detected;        /* MCX_detect::detectedphoton: all detections, including those beyond maxdetphotons */
    uint64_t saved;           /* MCX_detect::savedcount() */
    uint64_t launched;        /* photons processed */
    uint64_t steps;           /* voxel steps (MCX_photon::step calls; the fast kernels also count a step of length 0
                                 after a free-path draw of exactly 0, where the reference scatters without a step) */
    uint64_t crossings;       /* voxel changes (deposit sites) */
    uint64_t scatters;        /* scattering events */
    uint64_t reflections;     /* MCX_photon::reflect calls */
    uint64_t capped;          /* photons stopped by the per-photon step cap or the zero-progress guard (0 in a
                                 normal run) */
    float kernel_ms;          /* device time of the propagation kernel (CUDA events) */
    float total_ms;           /* wall time of the whole call */
    int32_t status;           /* same as the return value */
    int32_t block_size;       /* threads per CTA of the propagation launch */
    int32_t grid_size;        /* CTAs of the propagation launch */
    int32_t reserved;
} umcx_result;

/* Launch tuning; zero fields mean "choose automatically" (autotuner cache or built-in default). */
typedef struct umcx_tuning {
    int32_t block_size;       /* threads per CTA */
    int32_t blocks_per_sm;    /* resident CTAs per SM for the persistent grid */
    int32_t aggregation;      /* 0 auto, 1 plain atomics, 2 warp match-any aggregation of fluence adds */
    int32_t budget_ms;        /* wall-clock budget of one propagation launch; 0 = 300 000 ms.  When it runs out the
                                 kernel stops, the call returns UMCX_ERR_TIMEOUT and the context stays usable. */
    int32_t grid_size;        /* CTAs of the launch; 0 = SM count x resident CTAs (one persistent wave).  A larger
                                 grid is allowed: its later CTAs start as earlier ones finish.  The reference's
                                 Session.ThreadNum / Session.BlockSize (-t / -T, L739-741) set it through
                                 umcx_job_tuning. */
    int32_t reserved;         /* 0 */
} umcx_tuning;

typedef struct umcx_context umcx_context;

/* library ABI version (UMCX_ABI_VERSION) */
int umcx_abi_version(void);
/* 1 when the library was built with device bounds checks (UMCX_DEVICE_CHECKS=1: every indexed device-buffer access
 * is tested first; a failing access is skipped and the call returns UMCX_ERR_CUDA naming it), else 0. */
int umcx_device_checks(void);

/* Create a context bound to CUDA device `device` (0-based; the reference's DeviceID is 1-based, L739). */
int umcx_create(umcx_context** ctx, int device);
void umcx_destroy(umcx_context* ctx);
/* Message of the last failure on ctx (empty string if none).  Valid until the next call on ctx. */
const char* umcx_last_error(const umcx_context* ctx);
/* Set the launch tuning used by later calls on ctx (NULL resets to automatic). */
int umcx_set_tuning(umcx_context* ctx, const umcx_tuning* tuning);

/* The four session seeds for RNGSeed (L724-727): srand(seed) then four rand() calls of the C library;
 * rngseed <= 0 uses the current time like the reference. */
int umcx_seeds_from_rngseed(int32_t rngseed, uint32_t seeds[4]);

/* Number of float columns of one detected-photon record (L157). */
int umcx_detp_columns(const umcx_sim* sim);

/*
 * Forward simulation with HOST buffers (replaces MCX_kernel, L722-781).
 *   labels   uint8 [nx][ny][nz] (z fastest), bit 7 = detector voxel
 *   media    float [mediumnum][4] = {mua, mus, g, n}, per-voxel units
 *   detpos   float [detnum][4]    = {x, y, z, radius} in voxels (may be NULL when detnum == 0)
 *   fluence  float [maxgate][nx][ny][nz], overwritten (may be NULL when issavevol == 0)
 *   detp     float [maxdetphotons][umcx_detp_columns(sim)] (may be NULL when issavedet == 0)
 * Copies in, runs the persistent propagation kernel, copies out, synchronises.  Device memory held by ctx and
 * reused by later calls: the label and output volumes, the detected-photon buffer, and unless UMCX_SIM_FP32_ACCUM
 * the FP64 accumulation volume (8 bytes per output element) plus up to 32 MB of copies of its hot part.
 */
int umcx_gpu_forward(umcx_context* ctx, const umcx_sim* sim, const uint8_t* labels, const float* media,
                     const float* detpos, float* fluence, float* detp, umcx_result* res);

/*
 * Forward simulation with DEVICE buffers d_labels, d_fluence, d_detp (same layouts as above; media and
 * detpos are host arrays) on `stream` (a cudaStream_t, NULL = legacy default stream).  Synchronises the
 * stream before returning and fills res.
 */
int umcx_gpu_forward_device(umcx_context* ctx, const umcx_sim* sim, const uint8_t* d_labels, const float* media,
                            const float* detpos, float* d_fluence, float* d_detp, void* stream, umcx_result* res);

/*
 * Differentiation (no counterpart in the reference, which has no adjoint and no photon replay).
 *
 * umcx_gpu_forward_adjoint runs the forward simulation (same inputs/outputs as umcx_gpu_forward) and additionally
 * keeps, inside the context: one extended record per detected photon (photon index = its replay seed, detector,
 * exit weight and time, path length and scatter count per label) and per-label tallies of the derivatives of the
 * summed output volume.  umcx_gpu_backward then reduces them (FP64) into derivatives with respect to every label's
 * mua and mus (per-voxel units, as in the media table), and optionally replays every detected photon from its seed
 * to build the voxel-wise mua Jacobian of each detector.  Readings are raw sums of exit weights (divide by the
 * launched photon count, or multiply by the normaliser, as needed); the time gate of a record is that of its exit
 * time.
 */
typedef struct umcx_adjoint {
    double* readings;        /* [detnum][maxgate]: sum of exit weights of detected photons, or NULL */
    double* dread_dmua;      /* [detnum][maxgate][mediumnum], or NULL */
    double* dread_dmus;      /* [detnum][maxgate][mediumnum], or NULL */
    double* dflu_dmua;       /* [mediumnum]: derivative of the sum of the raw output volume, or NULL */
    double* dflu_dmus;       /* [mediumnum], or NULL */
    float* jacobian;         /* [detnum][nx][ny][nz]: d(sum over gates of readings)/d(mua of the voxel); NULL skips
                                the replay */
    uint64_t records;        /* out: detected-photon records used */
    uint64_t replay_mismatch;/* out: replayed photons whose exit weight or detector differed from the record */
    float replay_ms;         /* out: device time of the replay kernel */
    int32_t reserved;
} umcx_adjoint;

int umcx_gpu_forward_adjoint(umcx_context* ctx, const umcx_sim* sim, const uint8_t* labels, const float* media,
                             const float* detpos, float* fluence, float* detp, umcx_result* res);
int umcx_gpu_backward(umcx_context* ctx, umcx_adjoint* out);

/*
 * Batched simulations (no counterpart in the reference): many independent forward simulations -- different grid
 * sizes, label counts, optics, sources and photon budgets -- run by one persistent kernel launch, replayed from a
 * CUDA graph captured at creation.  Each simulation's photons are seeded exactly as in a single run of it, so every
 * photon history, tally and output equals umcx_gpu_forward's for that simulation (up to the summation order of the
 * output volume).  A simulation with issavedet keeps its own detected-photon records (up to its maxdetphotons
 * rows of umcx_detp_columns(sim) floats, L164-176), from its own detectors detpos[i] ([detnum][4] {x, y, z, r};
 * detpos, or its entry, may be NULL for simulations that save no records).
 *
 * umcx_batch_create copies the host labels (uint8 [nx][ny][nz] each), media tables and detectors, allocates the
 * output and record pools and captures the graph (memsets, one or more kernel launches -- simulations are split into
 * launches only when their descriptors, optical and detector tables exceed a CTA's shared memory -- and the
 * FP64-to-FP32 rounding).  With labels NULL
 * the batch's label pool starts zeroed and the caller writes each simulation's labels in place before the first run,
 * at umcx_batch_labels(b, i) (for example with umcx_gpu_build_labels, no host copy at all).
 */
typedef struct umcx_batch umcx_batch;
int umcx_batch_create(umcx_context* ctx, int nsim, const umcx_sim* sims, const uint8_t* const* labels,
                      const float* const* media, const float* const* detpos, umcx_batch** out);
/* Device address of simulation i's uint8 label volume inside the batch's pool (NULL on a bad index). */
uint8_t* umcx_batch_labels(umcx_batch* b, int i);
/* Run the whole batch once (graph launch + synchronise).  total receives the summed tallies, event counts and
 * detections and kernel_ms the device time of the graph. */
int umcx_batch_run(umcx_batch* b, umcx_result* total);
/* Copy simulation i's output volume of the last run to fluence (host, [maxgate][nx][ny][nz]) and its detected-photon
 * records to detp (host, [saved][umcx_detp_columns]); res receives its energy_escape / energy_total / launched /
 * detected / saved.  Each of fluence, detp and res may be NULL. */
int umcx_batch_get(umcx_batch* b, int i, float* fluence, float* detp, umcx_result* res);
/* Re-time the batch with the given tuning (NULL: defaults) and re-capture its graph. */
int umcx_batch_set_tuning(umcx_batch* b, const umcx_tuning* tuning);
void umcx_batch_destroy(umcx_batch* b);

/*
 * Autotuner (no reference counterpart): times short runs (sim's photons scaled by `fraction`, at least 20 000) of
 * the forward kernel over block sizes and fluence-aggregation modes (per candidate a warm-up run, then the fastest
 * of three), keeps the fastest in *best and installs it on ctx.  Device buffers as for umcx_gpu_forward_device.
 */
int umcx_autotune(umcx_context* ctx, const umcx_sim* sim, const uint8_t* d_labels, const float* media,
                  const float* detpos, float* d_fluence, float* d_detp, double fraction, umcx_tuning* best,
                  float* best_ms);

/*
 * Device label builder (MCX_userio::initdomain, L537-604, and maskdetectors, L605-632, on the GPU; no reference
 * counterpart as an entry point).  The domain is either a list of compiled shape constructs painted over a Grid fill
 * value, or a host int32 volume (decoded JData input); detectors are then masked (bit 7) and the labels written as
 * uint8 into d_labels (device, dim[0]*dim[1]*dim[2] bytes) -- the same bytes the host front end produces.  Every
 * float comparison is evaluated with single roundings in the reference's order, so voxel-centre ties resolve as on
 * the host.  Synchronous on ctx's stream.  A shape value the reference would read from a missing key gives
 * UMCX_ERR_INPUT "type must be number, but is null"; a label without a medium gives UMCX_ERR_INPUT.
 */
enum { UMCX_SHAPE_SPHERE = 0, UMCX_SHAPE_BOX = 1, UMCX_SHAPE_XLAYER = 2, UMCX_SHAPE_YLAYER = 3, UMCX_SHAPE_ZLAYER = 4,
       UMCX_SHAPE_CYLINDER = 5 };
#define UMCX_SHAPE_HAS_TAG 0x1u   /* tag present (a shape that contains a voxel reads it) */
#define UMCX_SHAPE_HAS_SIZE0 0x2u /* Box "Sip.ze" components present: 0x2, 0x4, 0x8 */
#define UMCX_SHAPE_HAS_HI 0x10u   /* layer upper bound present */
typedef struct umcx_shape_op {    /* one shape, or one layer of a layers construct (48 bytes) */
    int32_t kind;                 /* UMCX_SHAPE_* */
    int32_t tag;
    uint32_t present;             /* UMCX_SHAPE_HAS_* bits */
    float f[8];                   /* sphere: O[3], R; box: O[3], Sip.ze[3]; layer: lo, hi; cylinder: C0[3],
                                     unit axis[3], squared axis length, R */
    int32_t reserved;
} umcx_shape_op;
typedef struct umcx_domain {
    uint32_t dim[3];
    int32_t fill;                 /* Grid Tag: every voxel's label before the shapes */
    const umcx_shape_op* ops;     /* shapes in input order (layers expanded in order) */
    int32_t nops;
    int32_t mediumnum;            /* labels must be < mediumnum */
    const int32_t* volume;        /* host int32 volume [nx][ny][nz] used instead of fill + ops, or NULL */
    const float* detpos;          /* [detnum][4] detector x, y, z, R (grid units) */
    int32_t detnum;
    int32_t reserved;
} umcx_domain;
int umcx_gpu_build_labels(umcx_context* ctx, const umcx_domain* dom, uint8_t* d_labels);

/*
 * Debug known-answer hook for the random number generator (MCX_rand, L187-215): for photons
 * photon_offset .. photon_offset+nphoton-1 of sim, writes `ndraw` consecutive rand01() values of each photon
 * to out[nphoton][ndraw] (host buffer), computed on the device.
 */
int umcx_gpu_rng_dump(umcx_context* ctx, const uint32_t seeds[4], uint64_t photon_offset, uint32_t nphoton,
                      uint32_t ndraw, float* out);

/*
 * Allocation-free forward simulation.  No counterpart in the reference.
 *
 * For callers that cannot call cudaMalloc (an application that owns the device memory pool and forbids foreign
 * allocations, a plugin living inside another framework's allocator, a real-time loop that must not allocate):
 * same inputs and outputs as umcx_gpu_forward_device (device buffers d_labels, d_fluence, d_detp; host arrays
 * media, detpos; a cudaStream_t), but no context, no allocation and no CUDA events.  The kernel's working state
 * (photon counter, tallies, optical table) lives in one fixed device array of UMCX_NOALLOC_SCRATCH_BYTES inside the
 * library, held by every GPU that loads it until the process exits; at most UMCX_NOALLOC_MAX_MEDIA media fit, and
 * larger tables are rejected with UMCX_ERR_INPUT.  The output volume is accumulated in FP32 directly in d_fluence
 * (as with UMCX_SIM_FP32_ACCUM).  Each call is synchronous: it reads the tallies back and synchronises its stream
 * before returning, so it cannot be recorded into a CUDA graph (stream capture).  The array's address belongs to
 * the device's primary context, so after the application resets the device (cudaDeviceReset) this entry point must
 * not be called again in the process.  All calls share the array: calls whose GPU work overlaps race and must be
 * serialised by the caller.  Inputs are checked by the same rules as umcx_gpu_forward_device.  res->kernel_ms is 0
 * (no events).
 */
#define UMCX_NOALLOC_SCRATCH_BYTES 8192
#define UMCX_NOALLOC_MAX_MEDIA 128
int umcx_gpu_forward_noalloc(int device, const umcx_sim* sim, const uint8_t* d_labels, const float* media,
                             const float* detpos, float* d_fluence, float* d_detp, void* stream, umcx_result* res);

/* Roofline denominators measured on the device (no reference counterpart): FP32 FMA instructions per second,
 * SFU (MUFU) operations per second and scattered float atomicAdd operations per second into an L2-resident array. */
typedef struct umcx_peaks {
    double fp32_fma_per_s;
    double sfu_per_s;
    double l2_atomic_per_s;
    int32_t sm_count;
    int32_t sm_clock_khz;
} umcx_peaks;
int umcx_measure_peaks(int device, umcx_peaks* out);

/* Command-line and JSON entry points of the reference (L850-856), running the simulation on the GPU and
 * writing the same console line and output files.  They return 0 on success and non-zero on failure. */
int MCX_run_cmd(char* argv[], int argn);
int MCX_run_json(char* jsoninput);

#ifdef __cplusplus
}
#endif

#endif /* UMCX_GPU_H */
