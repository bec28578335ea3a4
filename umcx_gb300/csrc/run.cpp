// run.cpp - the reference's driver, MCX_run_simulation (fangq/umcx src/umcx.cpp:783-848), on top of the GPU
// library, plus its C entry points MCX_run_cmd / MCX_run_json (L850-856) and the job API of umcx_host.h.
#include <chrono>
#include <cstdio>
#include <cstring>
#include <exception>
#include <memory>
#include <string>
#include <vector>

#include "../../include/umcx_gpu.h"
#include "../../include/umcx_host.h"
#include "frontend.h"

using umcx::Action;
using umcx::Job;
using umcx::UserIO;

struct umcx_job {
    std::unique_ptr<UserIO> io;
    Job job;
    std::string err;
    std::string console;
    int action = 0;
};

namespace {

int device_from(const UserIO& io) {
    const umcx::js::Value* s = io.cfg.find("Session");
    int dev = 1;
    if (s && s->contains("DeviceID")) dev = s->at("DeviceID").as_int();
    return dev > 0 ? dev - 1 : 0;  // DeviceID is 1-based (L739)
}

// MCX_run_simulation (L783-848): parse, simulate, print the summary line, write outputs.  Returns 0 on success.
int run_simulation(int argc, const char* const argv[], std::string* errmsg) {
    try {
        UserIO io(argc, argv);
        if (io.action == Action::Help || io.action == Action::DumpJson) {
            std::fputs(io.console.c_str(), stdout);
            std::fflush(stdout);
            return 0;
        }
        if (io.action == Action::DumpMask) {
            const std::string id = io.session_id();
            io.save_volume_i32(io.domain, id.empty() ? std::string("vol.bnii") : id + "_vol.bnii");
            return 0;
        }
        Job job = umcx::make_job(io);
        const umcx_sim& s = job.sim;
        umcx_context* ctx = nullptr;
        int rc = umcx_create(&ctx, device_from(io));
        if (rc != UMCX_OK) throw std::runtime_error("no usable CUDA device for the simulation");
        std::unique_ptr<umcx_context, void (*)(umcx_context*)> guard(ctx, umcx_destroy);
        if ((job.tuning.block_size || job.tuning.grid_size) && umcx_set_tuning(ctx, &job.tuning) != UMCX_OK)
            throw std::runtime_error(std::string("invalid launch shape: ") + umcx_last_error(ctx));

        const auto t0 = std::chrono::steady_clock::now();  // MCX_clock at L812 (includes transfers)
        const size_t nout = 1ULL * s.dim[0] * s.dim[1] * s.dim[2] * s.dim[3];
        const int cols = umcx_detp_columns(&s);
        std::vector<float> fluence(s.issavevol ? nout : 0);
        std::vector<float> detp(s.issavedet ? static_cast<size_t>(s.maxdetphotons) * cols : 0);
        umcx_result res;
        std::memset(&res, 0, sizeof(res));
        rc = umcx_gpu_forward(ctx, &s, job.labels.data(), job.media.data(), job.detpos.data(),
                              fluence.empty() ? nullptr : fluence.data(), detp.empty() ? nullptr : detp.data(), &res);
        if (rc != UMCX_OK) throw std::runtime_error(std::string("GPU simulation failed: ") + umcx_last_error(ctx));
        const double energyescape = res.energy_escape, energytotal = res.energy_total;
        const float normalizer = job.normalizer_for(energytotal);
        const double elapsed = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        std::printf(
            "simulated energy %.2f, speed %.2f photon/ms, duration %.6f ms, normalizer %.6f, detected %d, absorbed "
            "%.6f%%\n",
            energytotal, static_cast<double>(s.nphoton) / elapsed, elapsed, normalizer, static_cast<int>(res.saved),
            (energytotal - energyescape) / energytotal * 100.);
        std::fflush(stdout);
        const std::string id = io.session_id();
        if (s.issavevol) {
            if (job.isnormalized && normalizer != 1.f)
                for (float& v : fluence) v *= normalizer;  // MCX_volume::scale (L141-145)
            io.save_volume_f32(fluence, s.dim, id.empty() ? std::string("output.bnii") : id + ".bnii");
        }
        if (s.issavedet) {
            io.save_detphoton(detp, res.saved, res.detected, cols, s,
                              id.empty() ? std::string("output_detp.jdb") : id + "_detp.jdb");
        }
        return 0;
    } catch (const std::exception& e) {
        if (errmsg) *errmsg = e.what();
        return 1;
    }
}

}  // namespace

extern "C" {

int MCX_run_cmd(char* argv[], int argn) {
    std::string err;
    int rc = run_simulation(argn, argv, &err);
    if (rc) std::fprintf(stderr, "umcx encounters an error:\n%s\n", err.c_str());
    return rc;
}

int MCX_run_json(char* jsoninput) {
    const char* argv[] = {"", "--json", jsoninput};
    std::string err;
    int rc = run_simulation(3, argv, &err);
    if (rc) std::fprintf(stderr, "umcx encounters an error:\n%s\n", err.c_str());
    return rc;
}

int umcx_main(int argc, char* argv[]) {
    std::string err;
    int rc = run_simulation(argc, argv, &err);
    if (rc) {
        // the reference's main() prints to stdout and returns 1 (L868-875)
        std::printf("umcx encounters an error:\n%s\n", err.c_str());
        return 1;
    }
    return 0;
}

int umcx_job_from_args(umcx_job** out, int argc, const char* const argv[]) {
    return umcx_job_from_args_ex(out, argc, argv, 0u);
}

int umcx_job_from_args_ex(umcx_job** out, int argc, const char* const argv[], uint32_t flags) {
    if (!out) return UMCX_ERR_INPUT;
    *out = nullptr;
    umcx_job* j = new (std::nothrow) umcx_job();
    if (!j) return UMCX_ERR_INPUT;
    *out = j;
    if (flags & ~UMCX_JOB_DEVICE_LABELS) {
        j->err = "unknown umcx_job_from_args_ex flags";
        return UMCX_ERR_INPUT;
    }
    try {
        j->io.reset(new UserIO(argc, argv, (flags & UMCX_JOB_DEVICE_LABELS) != 0));
        j->action = static_cast<int>(j->io->action);
        j->console = j->io->console;
        if (j->io->action == Action::Run) j->job = umcx::make_job(*j->io);
        return UMCX_OK;
    } catch (const std::exception& e) {
        j->err = e.what();
        return UMCX_ERR_INPUT;
    }
}

int umcx_job_from_json(umcx_job** out, const char* json) {
    const char* argv[] = {"", "--json", json ? json : "{}"};
    return umcx_job_from_args(out, 3, argv);
}

void umcx_job_free(umcx_job* j) { delete j; }
const char* umcx_job_error(const umcx_job* j) { return j ? j->err.c_str() : "no job"; }
int umcx_job_action(const umcx_job* j) { return j ? j->action : -1; }
const char* umcx_job_console(const umcx_job* j) { return j ? j->console.c_str() : ""; }
const umcx_sim* umcx_job_sim(const umcx_job* j) { return j && j->io ? &j->job.sim : nullptr; }
const uint8_t* umcx_job_labels(const umcx_job* j) {
    return j && !j->job.labels.empty() ? j->job.labels.data() : nullptr;
}

int umcx_job_build_labels(const umcx_job* j, umcx_context* ctx, uint8_t* d_labels) {
    if (!j || !j->io || j->action != static_cast<int>(Action::Run) || !ctx || !d_labels) return UMCX_ERR_INPUT;
    const UserIO& io = *j->io;
    umcx_domain dom;
    std::memset(&dom, 0, sizeof(dom));
    dom.dim[0] = io.domain.nx;
    dom.dim[1] = io.domain.ny;
    dom.dim[2] = io.domain.nz;
    dom.fill = io.grid_fill;
    dom.ops = io.shape_ops.data();
    dom.nops = static_cast<int32_t>(io.shape_ops.size());
    dom.mediumnum = j->job.sim.mediumnum;
    dom.volume = io.domain_is_volume ? io.domain.vol.data() : nullptr;
    dom.detpos = j->job.detpos.data();
    dom.detnum = j->job.sim.detnum;
    return umcx_gpu_build_labels(ctx, &dom, d_labels);
}
int umcx_job_tuning(const umcx_job* j, umcx_tuning* out) {
    if (!j || !j->io || !out) return UMCX_ERR_INPUT;
    *out = j->job.tuning;
    return UMCX_OK;
}
const float* umcx_job_media(const umcx_job* j) { return j ? j->job.media.data() : nullptr; }
const float* umcx_job_detpos(const umcx_job* j) { return j ? j->job.detpos.data() : nullptr; }
int umcx_job_isnormalized(const umcx_job* j) { return j ? j->job.isnormalized : 0; }
float umcx_job_normalizer(const umcx_job* j, double energytotal) { return j ? j->job.normalizer_for(energytotal) : 0.f; }
const char* umcx_job_config_json(const umcx_job* j, int indent) {
    static thread_local std::string buf;
    buf = (j && j->io) ? j->io->cfg.dump(indent) : std::string();
    return buf.c_str();
}
int umcx_job_domain_int32(const umcx_job* j, int32_t* out, size_t n) {
    if (!j || !j->io || !out || j->io->domain_on_device) return UMCX_ERR_INPUT;
    if (n < j->io->domain.vol.size()) return UMCX_ERR_INPUT;
    std::memcpy(out, j->io->domain.vol.data(), j->io->domain.vol.size() * sizeof(int32_t));
    return UMCX_OK;
}
int umcx_job_domain_dims(const umcx_job* j, uint32_t dims[3]) {
    if (!j || !j->io || !dims) return UMCX_ERR_INPUT;
    dims[0] = j->io->domain.nx;
    dims[1] = j->io->domain.ny;
    dims[2] = j->io->domain.nz;
    return UMCX_OK;
}
int umcx_job_write_outputs(const umcx_job* j, const float* fluence, const float* detp, const umcx_result* res,
                           int normalize) {
    if (!j || !j->io || !res) return UMCX_ERR_INPUT;
    try {
        const umcx_sim& s = j->job.sim;
        const std::string id = j->io->session_id();
        if (s.issavevol && fluence) {
            const size_t nout = 1ULL * s.dim[0] * s.dim[1] * s.dim[2] * s.dim[3];
            std::vector<float> v(fluence, fluence + nout);
            const float norm = j->job.normalizer_for(res->energy_total);
            if (normalize && j->job.isnormalized && norm != 1.f)
                for (float& x : v) x *= norm;
            j->io->save_volume_f32(v, s.dim, id.empty() ? std::string("output.bnii") : id + ".bnii");
        }
        if (s.issavedet) {
            const int cols = umcx_detp_columns(&s);
            std::vector<float> rows(detp ? detp : nullptr, detp ? detp + res->saved * cols : nullptr);
            j->io->save_detphoton(rows, res->saved, res->detected, cols, s,
                                  id.empty() ? std::string("output_detp.jdb") : id + "_detp.jdb");
        }
        return UMCX_OK;
    } catch (const std::exception&) {
        return UMCX_ERR_INPUT;
    }
}
int umcx_job_dump_mask(const umcx_job* j, const char* path) {
    if (!j || !j->io || !path || j->io->domain_on_device) return UMCX_ERR_INPUT;
    try {
        j->io->save_volume_i32(j->io->domain, path);
        return UMCX_OK;
    } catch (const std::exception&) {
        return UMCX_ERR_INPUT;
    }
}

}  // extern "C"
