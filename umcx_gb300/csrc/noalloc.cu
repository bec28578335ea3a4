// noalloc.cu - a forward-simulation entry point that allocates no memory at all.
//
// Who needs it: callers that must not (or cannot) call cudaMalloc -- code running inside a host application that
// owns the GPU memory budget and forbids foreign allocations (a serving process with a fixed memory pool, a plugin
// loaded into another framework's allocator, a real-time loop where an allocation could block or fail late).  They
// bring their own device buffers for the inputs and outputs; the few bytes of working state the propagation kernel
// needs besides those (the photon counter, the energy and event tallies, the per-label optical table) live here in
// one fixed, file-scope device array instead of library allocations.
//
// The array is a static __device__ object: every GPU that loads this library holds it (SCRATCH_BYTES) until the
// process exits.  Host code cannot use its name as an address, so the first call on each device looks the address
// up with cudaGetSymbolAddress (with that device current) and caches it; make that first call before any stream
// capture.  All calls share the array and it keeps the last call's contents, so each call clears the counter and
// tallies before its launch.  Calls whose work overlaps on the GPU (different streams, or different host threads
// on the same device) race on the array and must be serialised by the caller.
#include <cuda_runtime.h>

#include <chrono>
#include <cstring>
#include <mutex>

#include "../../include/umcx_gpu.h"
#include "launch.h"
#include "propagate.cuh"

using namespace umcx_dev;

namespace {

// layout of the scratch array: [0, 128) tallies (KStats), [128, 136) photon counter, [256, ...) Medium table
constexpr size_t kStatsOff = 0;
constexpr size_t kCounterOff = 128;
constexpr size_t kMediaOff = 256;
constexpr size_t kScratchBytes = UMCX_NOALLOC_SCRATCH_BYTES;
static_assert(sizeof(KStats) <= kCounterOff, "tallies overlap the counter");
static_assert(kMediaOff + sizeof(Medium) * UMCX_NOALLOC_MAX_MEDIA <= kScratchBytes, "scratch too small");

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
unsigned char* g_scratch_ptr[kMaxDevices] = {};  // device address of g_scratch, per device

// once per device, with that device current: the device address of the scratch array
cudaError_t scratch_address(int device, unsigned char** out) {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess) return e;
        e = configure_fast_kernels();  // large dynamic shared memory for the per-thread partial paths
        if (e == cudaSuccess) e = configure_strict_kernels();
        if (e != cudaSuccess) return e;
        g_scratch_ptr[device] = static_cast<unsigned char*>(p);
    }
    *out = g_scratch_ptr[device];
    return cudaSuccess;
}

int fail(umcx_result* res, int code) {
    if (res) res->status = code;
    return code;
}

}  // namespace

extern "C" int umcx_gpu_forward_noalloc(int device, const umcx_sim* s, const uint8_t* d_labels, const float* media,
                                        const float* detpos, float* d_fluence, float* d_detp, void* stream,
                                        umcx_result* res) {
    const auto t0 = std::chrono::steady_clock::now();
    if (res) std::memset(res, 0, sizeof(*res));
    if (!s || !d_labels || !media || (s->detnum > 0 && !detpos)) return fail(res, UMCX_ERR_INPUT);
    if (s->flags & ~UMCX_SIM_FLAGS_ALL) return fail(res, UMCX_ERR_INPUT);
    for (int k = 0; k < 3; k++)
        if (s->dim[k] < 1 || s->dim[k] > 32767) return fail(res, UMCX_ERR_INPUT);
    if (s->dim[3] < 1 || s->dim[3] > UMCX_MAX_GATES) return fail(res, UMCX_ERR_INPUT);
    const unsigned long long nout = 1ULL * s->dim[0] * s->dim[1] * s->dim[2] * s->dim[3];
    if (nout >= (1ULL << 31)) return fail(res, UMCX_ERR_INPUT);
    // the optical table must fit the fixed scratch array
    if (s->mediumnum < 1 || s->mediumnum > UMCX_NOALLOC_MAX_MEDIA) return fail(res, UMCX_ERR_INPUT);
    if (s->detnum < 0 || s->detnum > UMCX_MAX_DET) return fail(res, UMCX_ERR_INPUT);
    if (s->srctype < 0 || s->srctype > 6 || !(s->rtstep > 0.f)) return fail(res, UMCX_ERR_INPUT);
    if (s->issavevol && !d_fluence) return fail(res, UMCX_ERR_INPUT);
    if (s->issavedet && s->maxdetphotons > 0 && !d_detp) return fail(res, UMCX_ERR_INPUT);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev || device >= kMaxDevices)
        return fail(res, UMCX_ERR_NODEV);
    if (cudaSetDevice(device) != cudaSuccess) return fail(res, UMCX_ERR_NODEV);
    unsigned char* scratch = nullptr;
    if (scratch_address(device, &scratch) != cudaSuccess) return fail(res, UMCX_ERR_CUDA);
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
        return fail(res, UMCX_ERR_CUDA);
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    // kernel parameters and the optical table (same derived constants as the allocating entry points)
    KParams P;
    std::memset(&P, 0, sizeof(P));
    P.nx = static_cast<int>(s->dim[0]);
    P.ny = static_cast<int>(s->dim[1]);
    P.nz = static_cast<int>(s->dim[2]);
    P.maxgate = static_cast<int>(s->dim[3]);
    P.dimyz = s->dim[1] * s->dim[2];
    P.dimxyz = P.dimyz * s->dim[0];
    P.nphoton = s->nphoton;
    P.photon_offset = s->photon_offset;
    P.tstart = s->tstart;
    P.tend = s->tend;
    P.rtstep = s->rtstep;
    P.unitinmm = s->unitinmm;
    P.isreflect = s->isreflect;
    P.issavevol = s->issavevol;
    P.issavedet = s->issavedet;
    P.savedetflag = s->savedetflag;
    P.mediumnum = s->mediumnum;
    P.outputtype = s->outputtype;
    P.detnum = s->detnum;
    P.srctype = s->srctype;
    P.maxdetphotons = s->issavedet ? s->maxdetphotons : 0u;
    P.cols = umcx_detp_columns(s);
    P.ppathlen = (s->issavedet && (s->savedetflag & UMCX_DET_PPATH)) ? s->mediumnum : 0;
    P.step_cap = kDefaultStepCap;
    for (int k = 0; k < 4; k++) P.seeds[k] = s->seeds[k];
    P.srcpos = make_float4(s->srcpos[0], s->srcpos[1], s->srcpos[2], 1.f);
    P.srcdir = make_float4(s->srcdir[0], s->srcdir[1], s->srcdir[2], 0.f);
    P.srcrdir = make_float4(1.f / s->srcdir[0], 1.f / s->srcdir[1], 1.f / s->srcdir[2], 0.f);
    P.srcparam1 = make_float4(s->srcparam1[0], s->srcparam1[1], s->srcparam1[2], s->srcparam1[3]);
    P.srcparam2 = make_float4(s->srcparam2[0], s->srcparam2[1], s->srcparam2[2], s->srcparam2[3]);
    P.budget_ns = 600ULL * 1000000000ULL;
    for (int d = 0; d < s->detnum; d++)
        P.det[d] = make_float4(detpos[4 * d], detpos[4 * d + 1], detpos[4 * d + 2], detpos[4 * d + 3]);
    Medium hm[UMCX_NOALLOC_MAX_MEDIA];
    for (int i = 0; i < s->mediumnum; i++) {
        const float mua = media[4 * i], mus = media[4 * i + 1], g = media[4 * i + 2], n = media[4 * i + 3];
        hm[i].a = make_float4(mua, mus, g, n);
        hm[i].b = make_float4(mus != 0.f ? 1.f / mus : 0.f, deposit_factor(mua, s->outputtype),
                              g != 0.f ? 1.f / (2.f * g) : 0.f, n * kOneOverC0);
        hm[i].c = make_float4(1.f - g * g, 1.f - g, 2.f * g, 1.f + g * g);
    }

    KBuffers B;
    std::memset(&B, 0, sizeof(B));
    B.labels = d_labels;
    B.fluence = d_fluence;  // FP32 accumulation straight into the caller's output (no FP64 volume)
    B.detp = d_detp;
    set_extents(B, 1ULL * s->dim[0] * s->dim[1] * s->dim[2], s->issavevol ? nout : 0,
                d_detp ? static_cast<unsigned long long>(s->maxdetphotons) * umcx_detp_columns(s) : 0, 0);
    B.media = reinterpret_cast<const Medium*>(scratch + kMediaOff);
    B.stats = reinterpret_cast<KStats*>(scratch + kStatsOff);
    B.counter = reinterpret_cast<unsigned long long*>(scratch + kCounterOff);

    umcx_tuning tune;
    std::memset(&tune, 0, sizeof(tune));
    LaunchChoice lc = choose_launch(device, sms, tune, s, P);
    P.aggregate = lc.aggregate;

    // the scratch keeps the previous call's contents: clear the counter and tallies, refresh the table
    if (cudaMemsetAsync(scratch, 0, kMediaOff, st) != cudaSuccess) return fail(res, UMCX_ERR_CUDA);
    if (cudaMemcpyAsync(scratch + kMediaOff, hm, sizeof(Medium) * s->mediumnum, cudaMemcpyHostToDevice, st) !=
        cudaSuccess)
        return fail(res, UMCX_ERR_CUDA);
    if (s->issavevol && cudaMemsetAsync(d_fluence, 0, nout * sizeof(float), st) != cudaSuccess)
        return fail(res, UMCX_ERR_CUDA);
    launch_forward(lc, P, B, st, (s->flags & UMCX_SIM_STRICT_MATH) != 0);
    if (cudaGetLastError() != cudaSuccess) return fail(res, UMCX_ERR_CUDA);
    KStats stats;
    if (cudaMemcpyAsync(&stats, scratch + kStatsOff, sizeof(stats), cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return fail(res, UMCX_ERR_CUDA);
    if (cudaStreamSynchronize(st) != cudaSuccess) return fail(res, UMCX_ERR_CUDA);
    // deadline reached, or (checked builds) a failed device bounds check
    const int rc = stats.error >= kCheckError ? UMCX_ERR_CUDA : (stats.error ? UMCX_ERR_TIMEOUT : UMCX_OK);
    if (res) {
        res->energy_escape = stats.escape;
        res->energy_total = stats.total;
        res->detected = stats.detected;
        const unsigned long long maxdet = s->issavedet ? s->maxdetphotons : 0u;
        res->saved = stats.detected < maxdet ? stats.detected : maxdet;
        res->launched = stats.launched;
        res->steps = stats.steps;
        res->crossings = stats.crossings;
        res->scatters = stats.scatters;
        res->reflections = stats.reflections;
        res->capped = stats.capped;
        res->kernel_ms = 0.f;  // no CUDA events are created on this path
        res->total_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
        res->status = rc;
    }
    return rc;
}
