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
// up with cudaGetSymbolAddress (with that device current) and caches it.  The cached address belongs to the
// device's primary context: after a cudaDeviceReset by the host application the entry point must not be called
// again in that process.  Every call is synchronous -- it reads the tallies back and synchronises its stream before
// it returns -- so no call can be recorded into a CUDA graph.  All calls share the array and it keeps the last
// call's contents, so each call clears the counter and tallies before its launch.  Calls whose work overlaps on the
// GPU (different streams, or different host threads on the same device) race on the array and must be serialised
// by the caller.
#include <cuda_runtime.h>

#include <chrono>
#include <cstring>
#include <mutex>

#include "../../include/umcx_gpu.h"
#include "launch.h"
#include "params.h"
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
    // the same input rules as every other entry point (params.h), plus the optical table's fit in the fixed array
    if (check_sim(s) || !d_labels || !media || (s->detnum > 0 && !detpos)) return fail(res, UMCX_ERR_INPUT);
    if (s->mediumnum > UMCX_NOALLOC_MAX_MEDIA) return fail(res, UMCX_ERR_INPUT);
    const unsigned long long nout = 1ULL * s->dim[0] * s->dim[1] * s->dim[2] * s->dim[3];
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

    // kernel parameters and the optical table: the helpers the allocating entry points use
    KParams P = make_params(s, detpos);
    Medium hm[UMCX_NOALLOC_MAX_MEDIA];
    for (int i = 0; i < s->mediumnum; i++) hm[i] = make_medium(media + 4 * i, s->outputtype);

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
        res->block_size = lc.block;
        res->grid_size = lc.grid;
    }
    return rc;
}
