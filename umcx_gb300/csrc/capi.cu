// capi.cu - C ABI of libumcx_gb300.so: contexts, device buffers, launch configuration and the forward entry
// points that replace MCX_kernel (fangq/umcx src/umcx.cpp:722-781).
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <new>
#include <string>

#include "../../include/umcx_gpu.h"
#include "launch.h"
#include "propagate.cuh"

using namespace umcx_dev;

namespace {

struct DevBuf {
    void* ptr = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes) {
        if (bytes <= cap && ptr) return cudaSuccess;
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        cap = 0;
        size_t want = bytes < 256 ? 256 : bytes;
        cudaError_t e = cudaMalloc(&ptr, want);
        if (e == cudaSuccess) cap = want;
        return e;
    }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        cap = 0;
    }
};

}  // namespace

struct umcx_context {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::string err;
    umcx_tuning tuning{};
    DevBuf labels, fluence, detp, media, stats, counter, scratch, accum64;
};

namespace {

struct CudaError : std::exception {
    std::string msg;
    explicit CudaError(std::string m) : msg(std::move(m)) {}
    const char* what() const noexcept override { return msg.c_str(); }
};
struct InputError : std::exception {
    std::string msg;
    explicit InputError(std::string m) : msg(std::move(m)) {}
    const char* what() const noexcept override { return msg.c_str(); }
};
struct BudgetError : std::exception {
    std::string msg;
    explicit BudgetError(std::string m) : msg(std::move(m)) {}
    const char* what() const noexcept override { return msg.c_str(); }
};

#define UMCX_CK(call)                                                                                          \
    do {                                                                                                       \
        cudaError_t e_ = (call);                                                                               \
        if (e_ != cudaSuccess) throw CudaError(std::string(#call) + ": " + cudaGetErrorString(e_));           \
    } while (0)

template <class F>
int guarded(umcx_context* ctx, F&& f) {
    try {
        if (ctx) ctx->err.clear();
        return f();
    } catch (const InputError& e) {
        if (ctx) ctx->err = e.what();
        return UMCX_ERR_INPUT;
    } catch (const CudaError& e) {
        if (ctx) ctx->err = e.what();
        return UMCX_ERR_CUDA;
    } catch (const BudgetError& e) {
        if (ctx) ctx->err = e.what();
        return UMCX_ERR_TIMEOUT;
    } catch (const std::bad_alloc&) {
        if (ctx) ctx->err = "host memory allocation failed";
        return UMCX_ERR_INPUT;
    } catch (const std::exception& e) {
        if (ctx) ctx->err = e.what();
        return UMCX_ERR_INPUT;
    } catch (...) {
        if (ctx) ctx->err = "unknown error";
        return UMCX_ERR_INPUT;
    }
}

void validate(const umcx_sim* s) {
    if (!s) throw InputError("sim is NULL");
    if (s->flags & ~UMCX_SIM_FLAGS_ALL) throw InputError("unknown bits in umcx_sim.flags");
    for (int k = 0; k < 3; k++)
        if (s->dim[k] < 1 || s->dim[k] > 32767) throw InputError("dim[0..2] must be in 1..32767");
    if (s->dim[3] < 1 || s->dim[3] > UMCX_MAX_GATES) throw InputError("dim[3] (time gates) must be in 1..65535");
    const unsigned long long nvox = 1ULL * s->dim[0] * s->dim[1] * s->dim[2];
    if (nvox * s->dim[3] >= (1ULL << 31)) throw InputError("voxels x gates must be below 2^31");
    if (s->mediumnum < 1 || s->mediumnum > UMCX_MAX_MEDIA) throw InputError("mediumnum must be in 1..128");
    if (s->detnum < 0 || s->detnum > UMCX_MAX_DET) throw InputError("detnum must be in 0..64");
    if (!(s->rtstep > 0.f) || !std::isfinite(s->tend)) throw InputError("invalid time window");
    if (s->srctype < 0 || s->srctype > 6) throw InputError("unknown source type");
}

Medium make_medium(const float* m) {
    Medium r;
    const float mua = m[0], mus = m[1], g = m[2], n = m[3];
    r.a = make_float4(mua, mus, g, n);
    r.b = make_float4(mus != 0.f ? 1.f / mus : 0.f, mua != 0.f ? 1.f / mua : 0.f, g != 0.f ? 1.f / (2.f * g) : 0.f,
                      n * kOneOverC0);
    r.c = make_float4(1.f - g * g, 1.f - g, 2.f * g, 1.f + g * g);
    return r;
}

KParams make_params(const umcx_sim* s, const float* detpos) {
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
    P.step_cap = 1u << 28;
    for (int k = 0; k < 4; k++) P.seeds[k] = s->seeds[k];
    P.srcpos = make_float4(s->srcpos[0], s->srcpos[1], s->srcpos[2], 1.f);
    P.srcdir = make_float4(s->srcdir[0], s->srcdir[1], s->srcdir[2], 0.f);
    P.srcrdir = make_float4(1.f / s->srcdir[0], 1.f / s->srcdir[1], 1.f / s->srcdir[2], 0.f);
    P.srcparam1 = make_float4(s->srcparam1[0], s->srcparam1[1], s->srcparam1[2], s->srcparam1[3]);
    P.srcparam2 = make_float4(s->srcparam2[0], s->srcparam2[1], s->srcparam2[2], s->srcparam2[3]);
    P.budget_ns = 600ULL * 1000000000ULL;  // 10 minutes
    for (int d = 0; d < s->detnum; d++)
        P.det[d] = make_float4(detpos[4 * d], detpos[4 * d + 1], detpos[4 * d + 2], detpos[4 * d + 3]);
    return P;
}

void set_device(umcx_context* ctx) { UMCX_CK(cudaSetDevice(ctx->device)); }

// Enqueue one forward simulation on `stream`: clears the tallies and the output, launches the propagation kernel
// between the context's two events.  All buffers are device buffers.
void enqueue_forward(umcx_context* ctx, const umcx_sim* s, const uint8_t* d_labels, const float* media,
                     const float* detpos, float* d_fluence, float* d_detp, cudaStream_t stream) {
    validate(s);
    if (s->detnum > 0 && !detpos) throw InputError("detpos is NULL but detnum > 0");
    if (!media) throw InputError("media is NULL");
    if (!d_labels) throw InputError("labels is NULL");
    if (s->issavevol && !d_fluence) throw InputError("fluence is NULL but issavevol is set");
    if (s->issavedet && s->maxdetphotons > 0 && !d_detp) throw InputError("detp is NULL but issavedet is set");
    KParams P = make_params(s, detpos);
    Medium hm[UMCX_MAX_MEDIA];
    for (int i = 0; i < s->mediumnum; i++) hm[i] = make_medium(media + 4 * i);

    UMCX_CK(ctx->media.ensure(sizeof(Medium) * UMCX_MAX_MEDIA));
    UMCX_CK(ctx->stats.ensure(sizeof(KStats)));
    UMCX_CK(ctx->counter.ensure(sizeof(unsigned long long)));
    UMCX_CK(cudaMemcpyAsync(ctx->media.ptr, hm, sizeof(Medium) * s->mediumnum, cudaMemcpyHostToDevice, stream));
    UMCX_CK(cudaMemsetAsync(ctx->stats.ptr, 0, sizeof(KStats), stream));
    UMCX_CK(cudaMemsetAsync(ctx->counter.ptr, 0, sizeof(unsigned long long), stream));
    const size_t nout = 1ULL * s->dim[0] * s->dim[1] * s->dim[2] * s->dim[3];
    const bool fp64 = s->issavevol && !(s->flags & UMCX_SIM_FP32_ACCUM);
    if (fp64) {
        UMCX_CK(ctx->accum64.ensure(nout * sizeof(double)));
        UMCX_CK(cudaMemsetAsync(ctx->accum64.ptr, 0, nout * sizeof(double), stream));
    } else if (s->issavevol) {
        UMCX_CK(cudaMemsetAsync(d_fluence, 0, nout * sizeof(float), stream));
    }

    KBuffers B;
    std::memset(&B, 0, sizeof(B));
    B.labels = d_labels;
    B.fluence = d_fluence;
    B.detp = d_detp;
    B.media = static_cast<const Medium*>(ctx->media.ptr);
    B.stats = static_cast<KStats*>(ctx->stats.ptr);
    B.counter = static_cast<unsigned long long*>(ctx->counter.ptr);
    B.fluence64 = fp64 ? static_cast<double*>(ctx->accum64.ptr) : nullptr;

    LaunchChoice lc = choose_launch(ctx->device, ctx->sm_count, ctx->tuning, s, P);
    P.aggregate = lc.aggregate;
    if (ctx->tuning.budget_ms > 0) P.budget_ns = static_cast<unsigned long long>(ctx->tuning.budget_ms) * 1000000ULL;
    UMCX_CK(cudaEventRecord(ctx->ev0, stream));
    launch_forward(lc, P, B, stream, (s->flags & UMCX_SIM_STRICT_MATH) != 0);
    UMCX_CK(cudaGetLastError());
    UMCX_CK(cudaEventRecord(ctx->ev1, stream));
    if (fp64) {  // round the FP64 accumulation to the FP32 output once
        launch_fp64_to_fp32(static_cast<const double*>(ctx->accum64.ptr), d_fluence, nout, ctx->sm_count, stream);
        UMCX_CK(cudaGetLastError());
    }
}

void collect(umcx_context* ctx, const umcx_sim* s, cudaStream_t stream, umcx_result* res) {
    KStats st;
    UMCX_CK(cudaMemcpyAsync(&st, ctx->stats.ptr, sizeof(st), cudaMemcpyDeviceToHost, stream));
    UMCX_CK(cudaStreamSynchronize(stream));
    float ms = 0.f;
    UMCX_CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    if (res) {
        res->energy_escape = st.escape;
        res->energy_total = st.total;
        res->detected = st.detected;
        const unsigned long long maxdet = s->issavedet ? s->maxdetphotons : 0u;
        res->saved = st.detected < maxdet ? st.detected : maxdet;
        res->launched = st.launched;
        res->steps = st.steps;
        res->crossings = st.crossings;
        res->scatters = st.scatters;
        res->reflections = st.reflections;
        res->capped = st.capped;
        res->kernel_ms = ms;
        res->status = st.error ? UMCX_ERR_TIMEOUT : UMCX_OK;
    }
    if (st.error) throw BudgetError("propagation kernel stopped at its wall-clock budget; results are partial");
}

}  // namespace

extern "C" {

int umcx_abi_version(void) { return UMCX_ABI_VERSION; }

int umcx_create(umcx_context** out, int device) {
    if (!out) return UMCX_ERR_INPUT;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) return UMCX_ERR_NODEV;
    if (device < 0 || device >= n) return UMCX_ERR_NODEV;
    umcx_context* ctx = new (std::nothrow) umcx_context();
    if (!ctx) return UMCX_ERR_INPUT;
    ctx->device = device;
    int rc = guarded(ctx, [&]() {
        set_device(ctx);
        UMCX_CK(cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device));
        UMCX_CK(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
        UMCX_CK(cudaEventCreate(&ctx->ev0));
        UMCX_CK(cudaEventCreate(&ctx->ev1));
        UMCX_CK(configure_fast_kernels());
        UMCX_CK(configure_strict_kernels());
        return UMCX_OK;
    });
    if (rc != UMCX_OK) {
        std::fprintf(stderr, "umcx_create: %s\n", ctx->err.c_str());
        umcx_destroy(ctx);
        return rc;
    }
    *out = ctx;
    return UMCX_OK;
}

void umcx_destroy(umcx_context* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    ctx->labels.release();
    ctx->fluence.release();
    ctx->detp.release();
    ctx->media.release();
    ctx->stats.release();
    ctx->counter.release();
    ctx->scratch.release();
    ctx->accum64.release();
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

const char* umcx_last_error(const umcx_context* ctx) { return ctx ? ctx->err.c_str() : "no context"; }

int umcx_set_tuning(umcx_context* ctx, const umcx_tuning* t) {
    if (!ctx) return UMCX_ERR_INPUT;
    return guarded(ctx, [&]() {
        if (!t) {
            std::memset(&ctx->tuning, 0, sizeof(ctx->tuning));
            return UMCX_OK;
        }
        if (t->block_size < 0 || t->block_size > 1024 || (t->block_size % 32) != 0)
            throw InputError("block_size must be a multiple of 32 in 0..1024");
        if (t->blocks_per_sm < 0 || t->blocks_per_sm > 32) throw InputError("blocks_per_sm must be in 0..32");
        if (t->aggregation < 0 || t->aggregation > 2) throw InputError("aggregation must be 0, 1 or 2");
        if (t->budget_ms < 0) throw InputError("budget_ms must be >= 0");
        ctx->tuning = *t;
        return UMCX_OK;
    });
}

int umcx_seeds_from_rngseed(int32_t rngseed, uint32_t seeds[4]) {
    if (!seeds) return UMCX_ERR_INPUT;
    // srand(seed) followed by four rand() calls of the C library (L724-727), through the reentrant interface so
    // the caller's own rand() state is left alone; rngseed <= 0 means "seed from the clock" like the reference
    unsigned seed = rngseed > 0 ? static_cast<unsigned>(rngseed) : static_cast<unsigned>(std::time(nullptr));
    struct random_data rd;
    char state[128];
    std::memset(&rd, 0, sizeof(rd));
    std::memset(state, 0, sizeof(state));
    if (initstate_r(seed, state, sizeof(state), &rd) != 0) return UMCX_ERR_INPUT;
    for (int i = 0; i < 4; i++) {
        int32_t v = 0;
        random_r(&rd, &v);
        seeds[i] = static_cast<uint32_t>(v);
    }
    return UMCX_OK;
}

int umcx_detp_columns(const umcx_sim* s) {
    if (!s) return 0;
    return (s->savedetflag & UMCX_DET_ID) + ((s->savedetflag & UMCX_DET_PPATH) > 0) * s->mediumnum +
           (((s->savedetflag & UMCX_DET_EXITPOS) > 0) + ((s->savedetflag & UMCX_DET_EXITDIR) > 0)) * 3;
}

int umcx_gpu_forward_device(umcx_context* ctx, const umcx_sim* s, const uint8_t* d_labels, const float* media,
                            const float* detpos, float* d_fluence, float* d_detp, void* stream, umcx_result* res) {
    if (!ctx) return UMCX_ERR_INPUT;
    auto t0 = std::chrono::steady_clock::now();
    int rc = guarded(ctx, [&]() {
        set_device(ctx);
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        enqueue_forward(ctx, s, d_labels, media, detpos, d_fluence, d_detp, st);
        collect(ctx, s, st, res);
        return UMCX_OK;
    });
    if (res) {
        res->total_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
        res->status = rc;
    }
    return rc;
}

int umcx_gpu_forward(umcx_context* ctx, const umcx_sim* s, const uint8_t* labels, const float* media,
                     const float* detpos, float* fluence, float* detp, umcx_result* res) {
    if (!ctx) return UMCX_ERR_INPUT;
    auto t0 = std::chrono::steady_clock::now();
    int rc = guarded(ctx, [&]() {
        set_device(ctx);
        validate(s);
        if (!labels) throw InputError("labels is NULL");
        cudaStream_t st = ctx->stream;
        const size_t nvox = 1ULL * s->dim[0] * s->dim[1] * s->dim[2];
        const size_t nout = nvox * s->dim[3];
        const int cols = umcx_detp_columns(s);
        const size_t ndet = (s->issavedet ? 1ULL * s->maxdetphotons : 0ULL) * static_cast<size_t>(cols);
        UMCX_CK(ctx->labels.ensure(nvox));
        if (s->issavevol) UMCX_CK(ctx->fluence.ensure(nout * sizeof(float)));
        if (ndet) UMCX_CK(ctx->detp.ensure(ndet * sizeof(float)));
        UMCX_CK(cudaMemcpyAsync(ctx->labels.ptr, labels, nvox, cudaMemcpyHostToDevice, st));
        enqueue_forward(ctx, s, static_cast<const uint8_t*>(ctx->labels.ptr), media, detpos,
                        s->issavevol ? static_cast<float*>(ctx->fluence.ptr) : nullptr,
                        ndet ? static_cast<float*>(ctx->detp.ptr) : nullptr, st);
        umcx_result tmp;
        umcx_result* r = res ? res : &tmp;
        collect(ctx, s, st, r);
        if (s->issavevol && fluence)
            UMCX_CK(cudaMemcpyAsync(fluence, ctx->fluence.ptr, nout * sizeof(float), cudaMemcpyDeviceToHost, st));
        if (ndet && detp && r->saved)
            UMCX_CK(cudaMemcpyAsync(detp, ctx->detp.ptr, r->saved * cols * sizeof(float), cudaMemcpyDeviceToHost, st));
        UMCX_CK(cudaStreamSynchronize(st));
        return UMCX_OK;
    });
    if (res) {
        res->total_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
        res->status = rc;
    }
    return rc;
}

int umcx_gpu_rng_dump(umcx_context* ctx, const uint32_t seeds[4], uint64_t photon_offset, uint32_t nphoton,
                      uint32_t ndraw, float* out) {
    if (!ctx) return UMCX_ERR_INPUT;
    return guarded(ctx, [&]() {
        if (!seeds || !out) throw InputError("seeds/out is NULL");
        if (1ULL * nphoton * ndraw > (1ULL << 28)) throw InputError("nphoton * ndraw too large");
        set_device(ctx);
        const size_t bytes = 1ULL * nphoton * ndraw * sizeof(float);
        UMCX_CK(ctx->scratch.ensure(bytes));
        if (bytes) {
            launch_rng_dump(seeds, photon_offset, nphoton, ndraw, static_cast<float*>(ctx->scratch.ptr), ctx->stream);
            UMCX_CK(cudaGetLastError());
            UMCX_CK(cudaMemcpyAsync(out, ctx->scratch.ptr, bytes, cudaMemcpyDeviceToHost, ctx->stream));
        }
        UMCX_CK(cudaStreamSynchronize(ctx->stream));
        return UMCX_OK;
    });
}

}  // extern "C"
