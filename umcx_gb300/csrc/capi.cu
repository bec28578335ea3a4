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
#include <vector>
#include <algorithm>

#include "../../include/umcx_gpu.h"
#include "launch.h"
#include "params.h"
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
    DevBuf raster, raster_ops, raster_coords;  // device label builder: int32 volume + marks + flags, ops, lattices
    int last_block = 0, last_grid = 0;  // launch shape of the last propagation launch (reported in umcx_result)
    // adjoint state kept between umcx_gpu_forward_adjoint and umcx_gpu_backward
    DevBuf detrec, detext, grad, jac;
    umcx_sim adj_sim{};
    std::vector<float> adj_media, adj_det;
    unsigned long long adj_records = 0;
    bool adj_valid = false;
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

// KStats::error of a finished launch is 0, UMCX_ERR_TIMEOUT (deadline reached) or kCheckError + site when a device
// bounds check of a checked build (UMCX_DEVICE_CHECKS) failed; the last is an error of this library, reported as such
int launch_status(int error) { return error >= kCheckError ? UMCX_ERR_CUDA : (error ? UMCX_ERR_TIMEOUT : UMCX_OK); }
void throw_if_check_failed(int error) {
    static const char* const kSites[] = {"label read", "medium of a label", "output deposit", "partial-path slot",
                                         "detected-photon row", "Jacobian add"};
    if (error < kCheckError) return;
    const int site = error - kCheckError;
    throw CudaError(std::string("device bounds check failed: ") + (site < 6 ? kSites[site] : "unknown access"));
}

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
    if (const char* why = check_sim(s)) throw InputError(why);
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
    for (int i = 0; i < s->mediumnum; i++) hm[i] = make_medium(media + 4 * i, s->outputtype);

    UMCX_CK(ctx->media.ensure(sizeof(Medium) * UMCX_MAX_MEDIA));
    UMCX_CK(ctx->stats.ensure(sizeof(KStats)));
    UMCX_CK(ctx->counter.ensure(sizeof(unsigned long long)));
    UMCX_CK(cudaMemcpyAsync(ctx->media.ptr, hm, sizeof(Medium) * s->mediumnum, cudaMemcpyHostToDevice, stream));
    UMCX_CK(cudaMemsetAsync(ctx->stats.ptr, 0, sizeof(KStats), stream));
    UMCX_CK(cudaMemsetAsync(ctx->counter.ptr, 0, sizeof(unsigned long long), stream));
    const size_t nout = 1ULL * s->dim[0] * s->dim[1] * s->dim[2] * s->dim[3];
    const bool fp64 = s->issavevol && !(s->flags & UMCX_SIM_FP32_ACCUM);
    if (s->issavevol && !fp64) UMCX_CK(cudaMemsetAsync(d_fluence, 0, nout * sizeof(float), stream));

    KBuffers B;
    std::memset(&B, 0, sizeof(B));
    B.labels = d_labels;
    B.fluence = d_fluence;
    B.detp = d_detp;
    set_extents(B, 1ULL * s->dim[0] * s->dim[1] * s->dim[2], s->issavevol ? nout : 0,
                d_detp ? static_cast<unsigned long long>(s->maxdetphotons) * umcx_detp_columns(s) : 0, 0);
    B.media = static_cast<const Medium*>(ctx->media.ptr);
    B.stats = static_cast<KStats*>(ctx->stats.ptr);
    B.counter = static_cast<unsigned long long*>(ctx->counter.ptr);

    LaunchChoice lc = choose_launch(ctx->device, ctx->sm_count, ctx->tuning, s, P);
    P.aggregate = lc.aggregate;
    // the FP64 accumulation volume with the copies of its hot part (accumulator_replicas)
    const Replicas reps = fp64 ? accumulator_replicas(1ULL * s->dim[0] * s->dim[1] * s->dim[2], s->dim[3])
                               : Replicas{1u, 0ULL};
    if (fp64) {
        const size_t n64 = nout + (reps.copies - 1) * reps.len;
        UMCX_CK(ctx->accum64.ensure(n64 * sizeof(double)));
        UMCX_CK(cudaMemsetAsync(ctx->accum64.ptr, 0, n64 * sizeof(double), stream));
        B.fluence64 = static_cast<double*>(ctx->accum64.ptr);
        P.rep_mask = reps.copies - 1;
        P.rep_len = static_cast<unsigned>(reps.len);
        lc.rep = reps.mode(nout);
    }
    ctx->last_block = lc.block;
    ctx->last_grid = lc.grid;
    if (ctx->tuning.budget_ms > 0) P.budget_ns = static_cast<unsigned long long>(ctx->tuning.budget_ms) * 1000000ULL;
    UMCX_CK(cudaEventRecord(ctx->ev0, stream));
    launch_forward(lc, P, B, stream, (s->flags & UMCX_SIM_STRICT_MATH) != 0);
    UMCX_CK(cudaGetLastError());
    UMCX_CK(cudaEventRecord(ctx->ev1, stream));
    if (fp64) {  // round the FP64 accumulation (the sum of its replicas) to the FP32 output once
        launch_fp64_to_fp32(static_cast<const double*>(ctx->accum64.ptr), d_fluence, nout, ctx->sm_count, stream,
                            reps);
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
        res->status = launch_status(st.error);
        res->block_size = ctx->last_block;
        res->grid_size = ctx->last_grid;
    }
    throw_if_check_failed(st.error);
    if (st.error) throw BudgetError("propagation kernel stopped at its wall-clock budget; results are partial");
}

}  // namespace

extern "C" {

int umcx_abi_version(void) { return UMCX_ABI_VERSION; }
int umcx_device_checks(void) { return UMCX_DEVICE_CHECKS != 0 ? 1 : 0; }

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
        UMCX_CK(configure_adjoint_kernels());
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
    ctx->raster.release();
    ctx->raster_ops.release();
    ctx->raster_coords.release();
    ctx->detrec.release();
    ctx->detext.release();
    ctx->grad.release();
    ctx->jac.release();
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
        if (t->grid_size < 0 || t->grid_size > (1 << 24)) throw InputError("grid_size must be in 0..2^24");
        ctx->tuning = *t;
        return UMCX_OK;
    });
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

int umcx_gpu_forward_adjoint(umcx_context* ctx, const umcx_sim* s, const uint8_t* labels, const float* media,
                             const float* detpos, float* fluence, float* detp, umcx_result* res) {
    if (!ctx) return UMCX_ERR_INPUT;
    auto t0 = std::chrono::steady_clock::now();
    int rc = guarded(ctx, [&]() {
        set_device(ctx);
        validate(s);
        if (!labels || !media) throw InputError("labels/media is NULL");
        if (s->detnum > 0 && !detpos) throw InputError("detpos is NULL but detnum > 0");
        if (s->flags & UMCX_SIM_STRICT_MATH) throw InputError("the adjoint runs the fast-math kernels only");
        cudaStream_t st = ctx->stream;
        const int K = s->mediumnum;
        const size_t nvox = 1ULL * s->dim[0] * s->dim[1] * s->dim[2];
        const size_t nout = nvox * s->dim[3];
        const int cols = umcx_detp_columns(s);
        const unsigned long long cap = s->issavedet ? s->maxdetphotons : 0u;
        UMCX_CK(ctx->labels.ensure(nvox));
        UMCX_CK(cudaMemcpyAsync(ctx->labels.ptr, labels, nvox, cudaMemcpyHostToDevice, st));
        if (s->issavevol) UMCX_CK(ctx->fluence.ensure(nout * sizeof(float)));
        if (cap * cols) UMCX_CK(ctx->detp.ensure(cap * cols * sizeof(float)));
        UMCX_CK(ctx->detrec.ensure((cap ? cap : 1) * sizeof(DetRecord)));
        UMCX_CK(ctx->detext.ensure((cap ? cap : 1) * 2 * K * sizeof(float)));
        UMCX_CK(ctx->grad.ensure(2 * K * sizeof(double)));
        UMCX_CK(ctx->media.ensure(sizeof(Medium) * UMCX_MAX_MEDIA));
        UMCX_CK(ctx->stats.ensure(sizeof(KStats)));
        UMCX_CK(ctx->counter.ensure(sizeof(unsigned long long)));
        KParams P = make_params(s, detpos);
        P.maxdetphotons = static_cast<unsigned>(cap);
        Medium hm[UMCX_MAX_MEDIA];
        for (int i = 0; i < K; i++) hm[i] = make_medium(media + 4 * i, s->outputtype);
        UMCX_CK(cudaMemcpyAsync(ctx->media.ptr, hm, sizeof(Medium) * K, cudaMemcpyHostToDevice, st));
        UMCX_CK(cudaMemsetAsync(ctx->stats.ptr, 0, sizeof(KStats), st));
        UMCX_CK(cudaMemsetAsync(ctx->counter.ptr, 0, sizeof(unsigned long long), st));
        UMCX_CK(cudaMemsetAsync(ctx->grad.ptr, 0, 2 * K * sizeof(double), st));
        const bool fp64 = s->issavevol && !(s->flags & UMCX_SIM_FP32_ACCUM);
        // the FP64 volume with the copies of its hot part, as for the forward pass (accumulator_replicas)
        const Replicas reps = fp64 ? accumulator_replicas(nvox, s->dim[3]) : Replicas{1u, 0ULL};
        if (fp64) {
            const size_t n64 = nout + (reps.copies - 1) * reps.len;
            UMCX_CK(ctx->accum64.ensure(n64 * sizeof(double)));
            UMCX_CK(cudaMemsetAsync(ctx->accum64.ptr, 0, n64 * sizeof(double), st));
            P.rep_mask = reps.copies - 1;
            P.rep_len = static_cast<unsigned>(reps.len);
        } else if (s->issavevol) {
            UMCX_CK(cudaMemsetAsync(ctx->fluence.ptr, 0, nout * sizeof(float), st));
        }
        KBuffers B;
        std::memset(&B, 0, sizeof(B));
        B.labels = static_cast<const uint8_t*>(ctx->labels.ptr);
        B.fluence = s->issavevol ? static_cast<float*>(ctx->fluence.ptr) : nullptr;
        B.fluence64 = fp64 ? static_cast<double*>(ctx->accum64.ptr) : nullptr;
        B.detp = (cap * cols) ? static_cast<float*>(ctx->detp.ptr) : nullptr;
        set_extents(B, nvox, s->issavevol ? nout : 0, static_cast<unsigned long long>(cap) * cols, 0);
        B.media = static_cast<const Medium*>(ctx->media.ptr);
        B.stats = static_cast<KStats*>(ctx->stats.ptr);
        B.counter = static_cast<unsigned long long*>(ctx->counter.ptr);
        B.detrec = static_cast<DetRecord*>(ctx->detrec.ptr);
        B.detext = static_cast<float*>(ctx->detext.ptr);
        B.grad = static_cast<double*>(ctx->grad.ptr);
        int block = ctx->tuning.block_size > 0 ? ctx->tuning.block_size : 1024;  // 1024: 2 % faster than 256
        size_t smem = adjoint_smem(P, block);
        while (smem > kMaxDynamicSmem && block > 32) {
            block /= 2;
            smem = adjoint_smem(P, block);
        }
        if (smem > kMaxDynamicSmem) throw InputError("too many media for the adjoint's per-thread tallies");
        int occ = adjoint_occupancy(s->isreflect != 0, block, smem);
        if (occ < 1) occ = 1;
        int grid = ctx->tuning.grid_size > 0 ? ctx->tuning.grid_size : ctx->sm_count * occ;
        const unsigned long long lanes = 1ULL * grid * block;
        if (s->nphoton < lanes) grid = static_cast<int>(std::max<unsigned long long>(1ULL, (s->nphoton + block - 1) / block));
        P.aggregate = 0;
        if (ctx->tuning.budget_ms > 0) P.budget_ns = static_cast<unsigned long long>(ctx->tuning.budget_ms) * 1000000ULL;
        UMCX_CK(cudaEventRecord(ctx->ev0, st));
        ctx->last_block = block;
        ctx->last_grid = grid;
        launch_adjoint(grid, block, smem, s->isreflect != 0, fp64 ? reps.mode(nout) : kRepNone, P, B, st);
        UMCX_CK(cudaGetLastError());
        UMCX_CK(cudaEventRecord(ctx->ev1, st));
        if (fp64) {
            launch_fp64_to_fp32(static_cast<const double*>(ctx->accum64.ptr), static_cast<float*>(ctx->fluence.ptr), nout,
                                ctx->sm_count, st, reps);
            UMCX_CK(cudaGetLastError());
        }
        umcx_result tmp;
        umcx_result* r = res ? res : &tmp;
        collect(ctx, s, st, r);
        if (s->issavevol && fluence)
            UMCX_CK(cudaMemcpyAsync(fluence, ctx->fluence.ptr, nout * sizeof(float), cudaMemcpyDeviceToHost, st));
        if (cap * cols && detp && r->saved)
            UMCX_CK(cudaMemcpyAsync(detp, ctx->detp.ptr, r->saved * cols * sizeof(float), cudaMemcpyDeviceToHost, st));
        UMCX_CK(cudaStreamSynchronize(st));
        ctx->adj_sim = *s;
        ctx->adj_media.assign(media, media + 4 * K);
        ctx->adj_det.assign(detpos ? detpos : media, detpos ? detpos + 4 * s->detnum : media);
        ctx->adj_records = r->saved;
        ctx->adj_valid = true;
        return UMCX_OK;
    });
    if (res) {
        res->total_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
        res->status = rc;
    }
    return rc;
}

int umcx_gpu_backward(umcx_context* ctx, umcx_adjoint* out) {
    if (!ctx) return UMCX_ERR_INPUT;
    return guarded(ctx, [&]() {
        if (!out) throw InputError("out is NULL");
        if (!ctx->adj_valid) throw InputError("umcx_gpu_backward needs a preceding umcx_gpu_forward_adjoint");
        set_device(ctx);
        cudaStream_t st = ctx->stream;
        const umcx_sim* s = &ctx->adj_sim;
        const int K = s->mediumnum;
        const size_t nvox = 1ULL * s->dim[0] * s->dim[1] * s->dim[2];
        const size_t ncell = static_cast<size_t>(s->detnum) * s->dim[3];
        KParams P = make_params(s, ctx->adj_det.data());
        const unsigned long long n = ctx->adj_records;
        // detector readings and derivatives
        const size_t rbytes = ncell * sizeof(double), gbytes = ncell * K * sizeof(double);
        UMCX_CK(ctx->scratch.ensure(rbytes + 2 * gbytes + 64));
        double* d_read = static_cast<double*>(ctx->scratch.ptr);
        double* d_gmua = d_read + ncell;
        double* d_gmus = d_gmua + ncell * K;
        UMCX_CK(cudaMemsetAsync(d_read, 0, rbytes + 2 * gbytes, st));
        launch_adjoint_reduce(P, static_cast<const DetRecord*>(ctx->detrec.ptr), static_cast<const float*>(ctx->detext.ptr),
                              n, static_cast<const Medium*>(ctx->media.ptr), d_read, d_gmua, d_gmus, ctx->sm_count, st);
        UMCX_CK(cudaGetLastError());
        if (out->readings) UMCX_CK(cudaMemcpyAsync(out->readings, d_read, rbytes, cudaMemcpyDeviceToHost, st));
        if (out->dread_dmua) UMCX_CK(cudaMemcpyAsync(out->dread_dmua, d_gmua, gbytes, cudaMemcpyDeviceToHost, st));
        if (out->dread_dmus) UMCX_CK(cudaMemcpyAsync(out->dread_dmus, d_gmus, gbytes, cudaMemcpyDeviceToHost, st));
        const double* g = static_cast<const double*>(ctx->grad.ptr);
        if (out->dflu_dmua) UMCX_CK(cudaMemcpyAsync(out->dflu_dmua, g, K * sizeof(double), cudaMemcpyDeviceToHost, st));
        if (out->dflu_dmus) UMCX_CK(cudaMemcpyAsync(out->dflu_dmus, g + K, K * sizeof(double), cudaMemcpyDeviceToHost, st));
        out->records = n;
        out->replay_mismatch = 0;
        out->replay_ms = 0.f;
        if (out->jacobian && s->detnum > 0) {
            const size_t jbytes = static_cast<size_t>(s->detnum) * nvox * sizeof(float);
            UMCX_CK(ctx->jac.ensure(jbytes));
            UMCX_CK(cudaMemsetAsync(ctx->jac.ptr, 0, jbytes, st));
            UMCX_CK(cudaMemsetAsync(ctx->stats.ptr, 0, sizeof(KStats), st));
            UMCX_CK(cudaMemsetAsync(ctx->counter.ptr, 0, sizeof(unsigned long long), st));
            KBuffers B;
            std::memset(&B, 0, sizeof(B));
            B.labels = static_cast<const uint8_t*>(ctx->labels.ptr);
            B.media = static_cast<const Medium*>(ctx->media.ptr);
            B.stats = static_cast<KStats*>(ctx->stats.ptr);
            B.counter = static_cast<unsigned long long*>(ctx->counter.ptr);
            B.replay_list = static_cast<const DetRecord*>(ctx->detrec.ptr);
            B.replay_count = n;
            B.jacobian = static_cast<float*>(ctx->jac.ptr);
            set_extents(B, nvox, 0, 0, static_cast<unsigned long long>(s->detnum) * nvox);
            const int block = 128;
            int grid = static_cast<int>(std::min<unsigned long long>((n + block - 1) / block, 8ULL * ctx->sm_count));
            if (grid < 1) grid = 1;
            UMCX_CK(cudaEventRecord(ctx->ev0, st));
            launch_replay(grid, block, s->isreflect != 0, P, B, st);
            UMCX_CK(cudaGetLastError());
            UMCX_CK(cudaEventRecord(ctx->ev1, st));
            KStats stats;
            UMCX_CK(cudaMemcpyAsync(&stats, ctx->stats.ptr, sizeof(stats), cudaMemcpyDeviceToHost, st));
            UMCX_CK(cudaMemcpyAsync(out->jacobian, ctx->jac.ptr, jbytes, cudaMemcpyDeviceToHost, st));
            UMCX_CK(cudaStreamSynchronize(st));
            UMCX_CK(cudaEventElapsedTime(&out->replay_ms, ctx->ev0, ctx->ev1));
            out->replay_mismatch = stats.capped;
            throw_if_check_failed(stats.error);
            if (stats.error) throw BudgetError("replay kernel stopped at its wall-clock budget");
        }
        UMCX_CK(cudaStreamSynchronize(st));
        return UMCX_OK;
    });
}

int umcx_gpu_build_labels(umcx_context* ctx, const umcx_domain* dom, uint8_t* d_labels) {
    if (!ctx) return UMCX_ERR_INPUT;
    return guarded(ctx, [&]() {
        if (!dom || !d_labels) throw InputError("domain or labels is NULL");
        for (int k = 0; k < 3; k++)
            if (dom->dim[k] < 1 || dom->dim[k] > 32767) throw InputError("domain dimensions must be between 1 and 32767");
        if (dom->nops < 0 || (dom->nops > 0 && !dom->ops)) throw InputError("shape ops missing");
        if (dom->mediumnum < 1 || dom->mediumnum > UMCX_MAX_MEDIA) throw InputError("mediumnum must be in [1, 128]");
        if (dom->detnum < 0 || dom->detnum > UMCX_MAX_DET || (dom->detnum > 0 && !dom->detpos))
            throw InputError("detnum must be in [0, 64] with detpos given");
        set_device(ctx);
        cudaStream_t st = ctx->stream;
        const unsigned long long n = 1ULL * dom->dim[0] * dom->dim[1] * dom->dim[2];
        // working buffer: int32 volume | marks (n bytes, rounded to 256) | flags: missing (u32), first bad index (u64)
        const size_t vbytes = n * sizeof(int32_t), mbytes = (n + 255) & ~255ULL;
        UMCX_CK(ctx->raster.ensure(vbytes + mbytes + 256));
        int32_t* vol = static_cast<int32_t*>(ctx->raster.ptr);
        uint8_t* mark = reinterpret_cast<uint8_t*>(vol) + vbytes;
        unsigned* missing = reinterpret_cast<unsigned*>(mark + mbytes);
        unsigned long long* first_bad = reinterpret_cast<unsigned long long*>(mark + mbytes + 8);
        const unsigned long long none = ~0ULL;
        UMCX_CK(cudaMemsetAsync(mark, 0, mbytes + 8, st));
        UMCX_CK(cudaMemcpyAsync(first_bad, &none, sizeof(none), cudaMemcpyHostToDevice, st));
        if (dom->volume) {
            UMCX_CK(cudaMemcpyAsync(vol, dom->volume, vbytes, cudaMemcpyHostToDevice, st));
        } else {
            if (dom->nops > 0) {
                UMCX_CK(ctx->raster_ops.ensure(sizeof(umcx_shape_op) * static_cast<size_t>(dom->nops)));
                UMCX_CK(cudaMemcpyAsync(ctx->raster_ops.ptr, dom->ops, sizeof(umcx_shape_op) * static_cast<size_t>(dom->nops),
                                        cudaMemcpyHostToDevice, st));
            }
            launch_raster(static_cast<const umcx_shape_op*>(ctx->raster_ops.ptr), dom->nops, dom->fill, dom->dim, vol,
                          missing, ctx->sm_count, st);
            UMCX_CK(cudaGetLastError());
        }
        // detector lattices (L607-609): the coordinates come from the reference's own float accumulation
        // (start = -R - 1 + centre, step 0.5, while <= R + 1 + centre), generated here in the same order
        std::vector<float> coords;
        std::vector<DetLattice> lat(static_cast<size_t>(dom->detnum));
        constexpr size_t kMaxSamplesPerAxis = 1u << 16;
        for (int d = 0; d < dom->detnum; d++) {
            const float* dp = dom->detpos + 4 * d;
            DetLattice& L = lat[static_cast<size_t>(d)];
            L.x = dp[0];
            L.y = dp[1];
            L.z = dp[2];
            L.r = dp[3];
            unsigned* offs[3] = {&L.xoff, &L.yoff, &L.zoff};
            unsigned* cnts[3] = {&L.nxs, &L.nys, &L.nzs};
            for (int a = 0; a < 3; a++) {
                const float radius = dp[3], c = dp[a];
                *offs[a] = static_cast<unsigned>(coords.size());
                size_t cnt = 0;
                for (float v = -radius - 1.f + c; v <= radius + 1.f + c; v += 0.5f) {
                    if (++cnt > kMaxSamplesPerAxis) throw InputError("detector radius too large to mask");
                    coords.push_back(v);
                }
                *cnts[a] = static_cast<unsigned>(cnt);
            }
        }
        if (!coords.empty()) {
            UMCX_CK(ctx->raster_coords.ensure(coords.size() * sizeof(float)));
            UMCX_CK(cudaMemcpyAsync(ctx->raster_coords.ptr, coords.data(), coords.size() * sizeof(float),
                                    cudaMemcpyHostToDevice, st));
            for (const DetLattice& L : lat) {
                launch_mask_det(vol, dom->dim, L, static_cast<const float*>(ctx->raster_coords.ptr), mark, ctx->sm_count,
                                st);
                UMCX_CK(cudaGetLastError());
            }
        }
        launch_finish_labels(vol, mark, n, dom->mediumnum, d_labels, first_bad, ctx->sm_count, st);
        UMCX_CK(cudaGetLastError());
        unsigned flags_miss = 0;
        unsigned long long bad = none;
        UMCX_CK(cudaMemcpyAsync(&flags_miss, missing, sizeof(flags_miss), cudaMemcpyDeviceToHost, st));
        UMCX_CK(cudaMemcpyAsync(&bad, first_bad, sizeof(bad), cudaMemcpyDeviceToHost, st));
        UMCX_CK(cudaStreamSynchronize(st));  // the host vectors above stay alive until the copies are done
        if (flags_miss) throw InputError("type must be number, but is null");
        if (bad != none) {
            int32_t v = 0;
            UMCX_CK(cudaMemcpy(&v, vol + bad, sizeof(v), cudaMemcpyDeviceToHost));
            throw InputError("label " + std::to_string(v & 0x7FFFFFFF) + " has no entry in Domain.Media");
        }
        return UMCX_OK;
    });
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

int umcx_autotune(umcx_context* ctx, const umcx_sim* s, const uint8_t* d_labels, const float* media,
                  const float* detpos, float* d_fluence, float* d_detp, double fraction, umcx_tuning* best,
                  float* best_ms) {
    if (!ctx) return UMCX_ERR_INPUT;
    return guarded(ctx, [&]() {
        validate(s);
        set_device(ctx);
        if (!(fraction > 0.0) || fraction > 1.0) throw InputError("fraction must be in (0, 1]");
        umcx_sim probe = *s;
        const double n = static_cast<double>(s->nphoton) * fraction;
        probe.nphoton = static_cast<uint64_t>(n < 20000.0 ? 20000.0 : n);
        if (probe.nphoton > s->nphoton) probe.nphoton = s->nphoton;
        const umcx_tuning saved = ctx->tuning;
        umcx_tuning keep = saved;
        float keep_ms = 1e30f;
        const int blocks[] = {128, 256, 512, 1024};
        for (int agg = 1; agg <= 2; agg++) {
            for (int bs : blocks) {
                umcx_tuning t = saved;
                t.block_size = bs;
                t.blocks_per_sm = 0;
                t.aggregation = agg;
                ctx->tuning = t;
                // one warm-up run, then the fastest of three: the candidates differ by a few per cent, about the
                // spread of single runs (the launch drain varies from run to run)
                float ms = 1e30f;
                for (int rep = 0; rep < 4; rep++) {
                    umcx_result r;
                    enqueue_forward(ctx, &probe, d_labels, media, detpos, d_fluence, d_detp, ctx->stream);
                    collect(ctx, &probe, ctx->stream, &r);
                    if (rep > 0 && r.kernel_ms < ms) ms = r.kernel_ms;
                }
                if (ms < keep_ms) {
                    keep_ms = ms;
                    keep = t;
                }
            }
        }
        ctx->tuning = keep;
        if (best) *best = keep;
        if (best_ms) *best_ms = keep_ms;
        return UMCX_OK;
    });
}

}  // extern "C"

// ================================================================================================= batches
struct umcx_batch {
    umcx_context* ctx = nullptr;
    int nsim = 0;
    std::vector<umcx_sim> sims;
    std::vector<unsigned long long> out_off, label_off, detp_off;
    unsigned long long nout_total = 0, lab_total = 0, ndetp_total = 0;
    bool reflect = false, fp64 = true;
    struct Chunk {
        int first = 0, count = 0, media_first = 0, total_media = 0;
        int det_first = 0, total_det = 0, ppathlen = 0;  // detectors and partial-path slots of its simulations
        bool savedet = false;                             // some simulation of the chunk saves detected photons
        unsigned long long photons = 0, begin_off = 0;
        int block = 0, grid = 0;
        size_t smem = 0;
    };
    std::vector<Chunk> chunks;
    std::vector<SimDesc> descs;
    DevBuf labels, media, dets, d_descs, d_begin, tallies, out32, out64, detp, detected, counters, stats;
    cudaGraphExec_t exec = nullptr;
    umcx_tuning tuning{};
    std::vector<double> host_tallies;
    std::vector<unsigned long long> host_detected;
};

namespace {

constexpr size_t kBatchSmemBudget = 200 * 1024;

void batch_plan(umcx_batch* b) {
    for (auto& ch : b->chunks) {
        const int block = b->tuning.block_size > 0 ? b->tuning.block_size : 512;
        const size_t smem = batch_smem(ch.count, ch.total_media, ch.total_det, ch.ppathlen, block);
        if (smem > kMaxDynamicSmem) throw InputError("batch chunk does not fit shared memory at this block size");
        int occ = batch_occupancy(b->reflect, ch.savedet, block, smem);
        if (occ < 1) occ = 1;
        const int per_sm = b->tuning.blocks_per_sm > 0 ? std::min(b->tuning.blocks_per_sm, occ) : occ;
        int grid = b->ctx->sm_count * per_sm;
        if (ch.photons < 1ULL * grid * block)
            grid = static_cast<int>(std::max<unsigned long long>(1ULL, (ch.photons + block - 1) / block));
        ch.block = block;
        ch.grid = grid;
        ch.smem = smem;
    }
}

// enqueue one full batch run on the context stream (used inside the graph capture)
void batch_enqueue(umcx_batch* b, cudaStream_t st) {
    UMCX_CK(cudaMemsetAsync(b->stats.ptr, 0, sizeof(KStats), st));
    UMCX_CK(cudaMemsetAsync(b->counters.ptr, 0, sizeof(unsigned long long) * b->chunks.size(), st));
    UMCX_CK(cudaMemsetAsync(b->tallies.ptr, 0, sizeof(double) * 2 * b->nsim, st));
    UMCX_CK(cudaMemsetAsync(b->detected.ptr, 0, sizeof(unsigned long long) * b->nsim, st));
    if (b->fp64) UMCX_CK(cudaMemsetAsync(b->out64.ptr, 0, sizeof(double) * b->nout_total, st));
    else UMCX_CK(cudaMemsetAsync(b->out32.ptr, 0, sizeof(float) * b->nout_total, st));
    for (size_t c = 0; c < b->chunks.size(); c++) {
        const auto& ch = b->chunks[c];
        BParams bp;
        std::memset(&bp, 0, sizeof(bp));
        bp.sims = static_cast<const SimDesc*>(b->d_descs.ptr) + ch.first;
        bp.begin = static_cast<const unsigned long long*>(b->d_begin.ptr) + ch.begin_off;
        bp.tallies = static_cast<double*>(b->tallies.ptr) + 2 * ch.first;
        bp.dets = ch.total_det ? static_cast<const float4*>(b->dets.ptr) + ch.det_first : nullptr;
        bp.detected = static_cast<unsigned long long*>(b->detected.ptr) + ch.first;
        bp.nsim = ch.count;
        bp.total_media = ch.total_media;
        bp.total_det = ch.total_det;
        bp.ppathlen = ch.ppathlen;
        bp.savedet = ch.savedet ? 1 : 0;
        bp.aggregate = b->tuning.aggregation == 2 ? 1 : 0;
        bp.total = ch.photons;
        bp.budget_ns = b->tuning.budget_ms > 0 ? static_cast<unsigned long long>(b->tuning.budget_ms) * 1000000ULL
                                               : kDefaultBudgetNs;
        KBuffers B;
        std::memset(&B, 0, sizeof(B));
        B.labels = static_cast<const uint8_t*>(b->labels.ptr);
        B.fluence = static_cast<float*>(b->out32.ptr);
        B.fluence64 = b->fp64 ? static_cast<double*>(b->out64.ptr) : nullptr;
        B.detp = ch.savedet ? static_cast<float*>(b->detp.ptr) : nullptr;  // NULL when no simulation keeps rows
        set_extents(B, b->lab_total, b->nout_total, ch.savedet ? b->ndetp_total : 0, 0);
        B.media = static_cast<const Medium*>(b->media.ptr) + ch.media_first;
        B.stats = static_cast<KStats*>(b->stats.ptr);
        B.counter = static_cast<unsigned long long*>(b->counters.ptr) + c;
        launch_batch(ch.grid, ch.block, ch.smem, b->reflect, bp, B, st);
        UMCX_CK(cudaGetLastError());
    }
    if (b->fp64) {
        launch_fp64_to_fp32(static_cast<const double*>(b->out64.ptr), static_cast<float*>(b->out32.ptr), b->nout_total,
                            b->ctx->sm_count, st);
        UMCX_CK(cudaGetLastError());
    }
}

void batch_capture(umcx_batch* b) {
    if (b->exec) {
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
    batch_plan(b);
    cudaStream_t st = b->ctx->stream;
    UMCX_CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    try {
        batch_enqueue(b, st);
    } catch (...) {
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(st, &g);
        if (g) cudaGraphDestroy(g);
        throw;
    }
    cudaGraph_t graph = nullptr;
    UMCX_CK(cudaStreamEndCapture(st, &graph));
    cudaError_t e = cudaGraphInstantiate(&b->exec, graph, 0);
    cudaGraphDestroy(graph);
    UMCX_CK(e);
}

SimDesc make_desc(const umcx_sim* s, unsigned media_base, unsigned det_base, unsigned long long label_off,
                  unsigned long long out_off, unsigned long long detp_off) {
    const KParams P = make_params(s, nullptr);
    SimDesc d;
    std::memset(&d, 0, sizeof(d));
    d.nx = P.nx;
    d.ny = P.ny;
    d.nz = P.nz;
    d.maxgate = P.maxgate;
    d.dimyz = P.dimyz;
    d.dimxyz = P.dimxyz;
    d.isreflect = P.isreflect;
    d.issavevol = P.issavevol;
    d.outputtype = P.outputtype;
    d.srctype = P.srctype;
    d.det_base = det_base;
    d.media_base = media_base;
    d.tstart = P.tstart;
    d.tend = P.tend;
    d.rtstep = P.rtstep;
    d.unitinmm = P.unitinmm;
    for (int k = 0; k < 4; k++) d.seeds[k] = P.seeds[k];
    d.label_off = label_off;
    d.out_off = out_off;
    d.photon_offset = s->photon_offset;
    d.nphoton = s->nphoton;
    d.srcpos = P.srcpos;
    d.srcdir = P.srcdir;
    d.srcrdir = P.srcrdir;
    d.srcparam1 = P.srcparam1;
    d.srcparam2 = P.srcparam2;
    d.detnum = s->issavedet ? s->detnum : 0;
    d.savedetflag = P.savedetflag;
    d.ppathlen = P.ppathlen;
    d.cols = P.cols;
    d.maxdetphotons = P.maxdetphotons;
    d.detp_off = detp_off;
    return d;
}

// upload the begin (prefix) arrays of every chunk for photon counts `counts` (one per simulation)
void batch_upload_begin(umcx_batch* b, const std::vector<unsigned long long>& counts, DevBuf& dst,
                        std::vector<unsigned long long>* chunk_totals) {
    std::vector<unsigned long long> begin;
    if (chunk_totals) chunk_totals->clear();
    for (auto& ch : b->chunks) {
        unsigned long long acc = 0;
        for (int i = 0; i < ch.count; i++) {
            begin.push_back(acc);
            acc += counts[static_cast<size_t>(ch.first + i)];
        }
        begin.push_back(acc);
        if (chunk_totals) chunk_totals->push_back(acc);
    }
    UMCX_CK(dst.ensure(begin.size() * sizeof(unsigned long long)));
    UMCX_CK(cudaMemcpy(dst.ptr, begin.data(), begin.size() * sizeof(unsigned long long), cudaMemcpyHostToDevice));
}

}  // namespace

extern "C" {

int umcx_batch_create(umcx_context* ctx, int nsim, const umcx_sim* sims, const uint8_t* const* labels,
                      const float* const* media, const float* const* detpos, umcx_batch** out) {
    if (!ctx || !out) return UMCX_ERR_INPUT;
    *out = nullptr;
    umcx_batch* b = new (std::nothrow) umcx_batch();
    if (!b) return UMCX_ERR_INPUT;
    b->ctx = ctx;
    int rc = guarded(ctx, [&]() {
        if (nsim < 1 || !sims || !media) throw InputError("empty batch or NULL arrays");
        set_device(ctx);
        UMCX_CK(configure_batch_kernels());
        b->nsim = nsim;
        b->sims.assign(sims, sims + nsim);
        std::vector<Medium> table;
        std::vector<float4> dtable;
        std::vector<unsigned long long> label_off(static_cast<size_t>(nsim)), media_first(static_cast<size_t>(nsim)),
            det_first(static_cast<size_t>(nsim));
        unsigned long long lab_total = 0;
        b->out_off.resize(static_cast<size_t>(nsim));
        b->detp_off.resize(static_cast<size_t>(nsim));
        b->fp64 = false;
        for (int i = 0; i < nsim; i++) {
            const umcx_sim* s = &sims[i];
            validate(s);
            if (s->flags & UMCX_SIM_STRICT_MATH) throw InputError("batches run the fast-math kernel only");
            det_first[static_cast<size_t>(i)] = dtable.size();
            b->detp_off[static_cast<size_t>(i)] = b->ndetp_total;
            if (s->issavedet) {  // its detectors into the batch's table, its rows into the record pool
                if (s->detnum > 0 && (!detpos || !detpos[i]))
                    throw InputError("simulation " + std::to_string(i) + ": detpos is NULL but detnum > 0");
                const KParams P = make_params(s, detpos ? detpos[i] : nullptr);
                for (int d = 0; d < s->detnum; d++) dtable.push_back(P.det[d]);
                b->ndetp_total += static_cast<unsigned long long>(P.maxdetphotons) * static_cast<unsigned>(P.cols);
            }
            if ((labels && !labels[i]) || !media[i])
                throw InputError("simulation " + std::to_string(i) + ": NULL labels or media");
            const unsigned long long nvox = 1ULL * s->dim[0] * s->dim[1] * s->dim[2];
            label_off[static_cast<size_t>(i)] = lab_total;
            lab_total += (nvox + 15) & ~15ULL;
            b->out_off[static_cast<size_t>(i)] = b->nout_total;
            b->nout_total += s->issavevol ? nvox * s->dim[3] : 0;
            media_first[static_cast<size_t>(i)] = table.size();
            for (int m = 0; m < s->mediumnum; m++) table.push_back(make_medium(media[i] + 4 * m, s->outputtype));
            if (s->isreflect) b->reflect = true;
            if (s->issavevol && !(s->flags & UMCX_SIM_FP32_ACCUM)) b->fp64 = true;
        }
        // chunks: as many consecutive simulations as fit a CTA's shared memory at block 1024
        int first = 0;
        while (first < nsim) {
            umcx_batch::Chunk ch;
            ch.first = first;
            ch.media_first = static_cast<int>(media_first[static_cast<size_t>(first)]);
            ch.det_first = static_cast<int>(det_first[static_cast<size_t>(first)]);
            int count = 0, tm = 0, td = 0, pp = 0;
            while (first + count < nsim) {
                const umcx_sim& s = sims[first + count];
                const int dn = s.issavedet ? s.detnum : 0;
                const int pl = make_params(&s, nullptr).ppathlen;
                if (count > 0 && batch_smem(count + 1, tm + s.mediumnum, td + dn, std::max(pp, pl), 1024) > kBatchSmemBudget)
                    break;
                tm += s.mediumnum;
                td += dn;
                pp = std::max(pp, pl);
                if (s.issavedet) ch.savedet = true;
                count++;
            }
            ch.count = count;
            ch.total_media = tm;
            ch.total_det = td;
            ch.ppathlen = pp;
            b->chunks.push_back(ch);
            first += count;
        }
        // descriptors (media_base and det_base relative to the chunk's first medium and detector)
        b->descs.resize(static_cast<size_t>(nsim));
        for (auto& ch : b->chunks)
            for (int i = ch.first; i < ch.first + ch.count; i++) {
                const size_t k = static_cast<size_t>(i);
                b->descs[k] = make_desc(&sims[i], static_cast<unsigned>(media_first[k] - ch.media_first),
                                        static_cast<unsigned>(det_first[k] - ch.det_first), label_off[k],
                                        b->out_off[k], b->detp_off[k]);
            }
        std::vector<unsigned long long> counts(static_cast<size_t>(nsim)), totals;
        for (int i = 0; i < nsim; i++) counts[static_cast<size_t>(i)] = sims[i].nphoton;
        unsigned long long boff = 0;
        for (auto& ch : b->chunks) {
            ch.begin_off = boff;
            boff += static_cast<unsigned long long>(ch.count) + 1;
        }
        batch_upload_begin(b, counts, b->d_begin, &totals);
        for (size_t c = 0; c < b->chunks.size(); c++) b->chunks[c].photons = totals[c];
        // device buffers
        UMCX_CK(b->labels.ensure(lab_total));
        b->lab_total = lab_total;
        b->label_off = label_off;
        if (!labels) UMCX_CK(cudaMemset(b->labels.ptr, 0, lab_total));  // filled in place by the caller
        for (int i = 0; labels && i < nsim; i++) {
            const unsigned long long nvox = 1ULL * sims[i].dim[0] * sims[i].dim[1] * sims[i].dim[2];
            UMCX_CK(cudaMemcpy(static_cast<uint8_t*>(b->labels.ptr) + label_off[static_cast<size_t>(i)], labels[i], nvox,
                               cudaMemcpyHostToDevice));
        }
        UMCX_CK(b->media.ensure(table.size() * sizeof(Medium)));
        UMCX_CK(cudaMemcpy(b->media.ptr, table.data(), table.size() * sizeof(Medium), cudaMemcpyHostToDevice));
        UMCX_CK(b->d_descs.ensure(b->descs.size() * sizeof(SimDesc)));
        UMCX_CK(cudaMemcpy(b->d_descs.ptr, b->descs.data(), b->descs.size() * sizeof(SimDesc), cudaMemcpyHostToDevice));
        if (!dtable.empty()) {
            UMCX_CK(b->dets.ensure(dtable.size() * sizeof(float4)));
            UMCX_CK(cudaMemcpy(b->dets.ptr, dtable.data(), dtable.size() * sizeof(float4), cudaMemcpyHostToDevice));
        }
        if (b->ndetp_total) UMCX_CK(b->detp.ensure(sizeof(float) * b->ndetp_total));
        UMCX_CK(b->detected.ensure(sizeof(unsigned long long) * nsim));
        UMCX_CK(b->tallies.ensure(sizeof(double) * 2 * nsim));
        UMCX_CK(b->out32.ensure(sizeof(float) * (b->nout_total ? b->nout_total : 1)));
        if (b->fp64) UMCX_CK(b->out64.ensure(sizeof(double) * (b->nout_total ? b->nout_total : 1)));
        UMCX_CK(b->counters.ensure(sizeof(unsigned long long) * b->chunks.size()));
        UMCX_CK(b->stats.ensure(sizeof(KStats)));
        b->tuning = ctx->tuning;
        batch_capture(b);
        return UMCX_OK;
    });
    if (rc != UMCX_OK) {
        umcx_batch_destroy(b);
        return rc;
    }
    *out = b;
    return UMCX_OK;
}

int umcx_batch_run(umcx_batch* b, umcx_result* total) {
    if (!b) return UMCX_ERR_INPUT;
    umcx_context* ctx = b->ctx;
    auto t0 = std::chrono::steady_clock::now();
    int rc = guarded(ctx, [&]() {
        set_device(ctx);
        cudaStream_t st = ctx->stream;
        UMCX_CK(cudaEventRecord(ctx->ev0, st));
        UMCX_CK(cudaGraphLaunch(b->exec, st));
        UMCX_CK(cudaEventRecord(ctx->ev1, st));
        KStats stats;
        b->host_tallies.resize(static_cast<size_t>(2 * b->nsim));
        UMCX_CK(cudaMemcpyAsync(&stats, b->stats.ptr, sizeof(stats), cudaMemcpyDeviceToHost, st));
        UMCX_CK(cudaMemcpyAsync(b->host_tallies.data(), b->tallies.ptr, sizeof(double) * 2 * b->nsim,
                                cudaMemcpyDeviceToHost, st));
        b->host_detected.resize(static_cast<size_t>(b->nsim));
        UMCX_CK(cudaMemcpyAsync(b->host_detected.data(), b->detected.ptr, sizeof(unsigned long long) * b->nsim,
                                cudaMemcpyDeviceToHost, st));
        UMCX_CK(cudaStreamSynchronize(st));
        float ms = 0.f;
        UMCX_CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
        if (total) {
            std::memset(total, 0, sizeof(*total));
            for (int i = 0; i < b->nsim; i++) {
                const size_t k = static_cast<size_t>(i);
                total->energy_escape += b->host_tallies[2 * k];
                total->energy_total += b->host_tallies[2 * k + 1];
                total->detected += b->host_detected[k];
                total->saved += std::min<unsigned long long>(b->host_detected[k], b->descs[k].maxdetphotons);
            }
            total->launched = stats.launched;
            total->steps = stats.steps;
            total->crossings = stats.crossings;
            total->scatters = stats.scatters;
            total->reflections = stats.reflections;
            total->capped = stats.capped;
            total->kernel_ms = ms;
            total->status = launch_status(stats.error);
        }
        throw_if_check_failed(stats.error);
        if (stats.error) throw BudgetError("batched kernel stopped at its wall-clock budget; results are partial");
        return UMCX_OK;
    });
    if (total) {
        total->total_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
        total->status = rc;
    }
    return rc;
}

int umcx_batch_get(umcx_batch* b, int i, float* fluence, float* detp, umcx_result* res) {
    if (!b) return UMCX_ERR_INPUT;
    return guarded(b->ctx, [&]() {
        if (i < 0 || i >= b->nsim) throw InputError("simulation index out of range");
        set_device(b->ctx);
        const umcx_sim& s = b->sims[static_cast<size_t>(i)];
        if (fluence && s.issavevol) {
            const size_t n = 1ULL * s.dim[0] * s.dim[1] * s.dim[2] * s.dim[3];
            UMCX_CK(cudaMemcpy(fluence, static_cast<float*>(b->out32.ptr) + b->out_off[static_cast<size_t>(i)],
                               n * sizeof(float), cudaMemcpyDeviceToHost));
        }
        const SimDesc& d = b->descs[static_cast<size_t>(i)];
        const unsigned long long detected =
            b->host_detected.size() == static_cast<size_t>(b->nsim) ? b->host_detected[static_cast<size_t>(i)] : 0ULL;
        const unsigned long long saved = std::min<unsigned long long>(detected, d.maxdetphotons);
        if (detp && saved)
            UMCX_CK(cudaMemcpy(detp, static_cast<float*>(b->detp.ptr) + d.detp_off,
                               saved * static_cast<unsigned>(d.cols) * sizeof(float), cudaMemcpyDeviceToHost));
        if (res) {
            std::memset(res, 0, sizeof(*res));
            if (b->host_tallies.size() == static_cast<size_t>(2 * b->nsim)) {
                res->energy_escape = b->host_tallies[static_cast<size_t>(2 * i)];
                res->energy_total = b->host_tallies[static_cast<size_t>(2 * i + 1)];
            }
            res->launched = s.nphoton;
            res->detected = detected;
            res->saved = saved;
        }
        return UMCX_OK;
    });
}

int umcx_batch_set_tuning(umcx_batch* b, const umcx_tuning* t) {
    if (!b) return UMCX_ERR_INPUT;
    return guarded(b->ctx, [&]() {
        set_device(b->ctx);
        if (t) b->tuning = *t;
        else std::memset(&b->tuning, 0, sizeof(b->tuning));
        batch_capture(b);
        return UMCX_OK;
    });
}

uint8_t* umcx_batch_labels(umcx_batch* b, int i) {
    if (!b || i < 0 || i >= b->nsim || !b->labels.ptr) return nullptr;
    return static_cast<uint8_t*>(b->labels.ptr) + b->label_off[static_cast<size_t>(i)];
}

void umcx_batch_destroy(umcx_batch* b) {
    if (!b) return;
    cudaSetDevice(b->ctx->device);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    b->labels.release();
    b->media.release();
    b->d_descs.release();
    b->d_begin.release();
    b->tallies.release();
    b->dets.release();
    b->detp.release();
    b->detected.release();
    b->out32.release();
    b->out64.release();
    b->counters.release();
    b->stats.release();
    delete b;
}

}  // extern "C"
