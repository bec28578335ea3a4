/*
 * umcx_host.h - C ABI of the host front end in libumcx_gb300.so (no GPU needed for any of these calls).
 *
 * A "job" is a parsed reference-style input: what the reference's MCX_userio (fangq/umcx src/umcx.cpp:451-721)
 * builds from a command line or JSON, turned into the flat arrays the GPU entry points of umcx_gpu.h take
 * (MCX_run_simulation's set-up, L786-810).  umcx_job_build_labels is the one call here that uses the GPU.  Callers that already hold a label volume and a media table call
 * umcx_gpu_forward directly and never need a job.
 */
#ifndef UMCX_HOST_H
#define UMCX_HOST_H

#include <stddef.h>
#include <stdint.h>

#include "umcx_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct umcx_job umcx_job;

/* what the command line asked for (MCX_userio, L474-532) */
enum { UMCX_ACTION_RUN = 0, UMCX_ACTION_DUMPJSON = 1, UMCX_ACTION_DUMPMASK = 2, UMCX_ACTION_HELP = 3 };

/* Parse a reference command line (argv[0] = program name), L474-532.  On failure *job is still set (free it)
 * and umcx_job_error() holds the reference-style message. */
int umcx_job_from_args(umcx_job** job, int argc, const char* const argv[]);
/* Parse a JSON input string as MCX_run_json does (L853-856). */
int umcx_job_from_json(umcx_job** job, const char* json);
/* umcx_job_from_args with flags.  UMCX_JOB_DEVICE_LABELS: shape constructs are compiled but not painted and
 * detectors not masked on the host; umcx_job_labels returns NULL and the labels are made on the GPU by
 * umcx_job_build_labels (a missing shape value is then reported there instead of here). */
#define UMCX_JOB_DEVICE_LABELS 0x1u
int umcx_job_from_args_ex(umcx_job** job, int argc, const char* const argv[], uint32_t flags);
void umcx_job_free(umcx_job* job);
const char* umcx_job_error(const umcx_job* job);
int umcx_job_action(const umcx_job* job);
/* text the reference prints for help / --dumpjson */
const char* umcx_job_console(const umcx_job* job);
/* the merged configuration as JSON text (indent < 0: compact); valid until the next call on this thread */
const char* umcx_job_config_json(const umcx_job* job, int indent);

/* Simulation description and arrays for umcx_gpu_forward (valid while the job lives; only for UMCX_ACTION_RUN). */
const umcx_sim* umcx_job_sim(const umcx_job* job);
const uint8_t* umcx_job_labels(const umcx_job* job);
const float* umcx_job_media(const umcx_job* job);
const float* umcx_job_detpos(const umcx_job* job);
int umcx_job_isnormalized(const umcx_job* job);
/* Launch shape the input asks for (Session.BlockSize / ThreadNum, the -T / -t flags; L739-741): block_size and
 * grid_size set when either key is given, all zeros otherwise.  Pass it to umcx_set_tuning; the CLI and
 * MCX_run_cmd / MCX_run_json do. */
int umcx_job_tuning(const umcx_job* job, umcx_tuning* out);
/* output normaliser for a total launched energy (L820) */
float umcx_job_normalizer(const umcx_job* job, double energytotal);

/* Build the job's uint8 label volume on the GPU into d_labels (device, nx*ny*nz bytes) with
 * umcx_gpu_build_labels: shapes painted over the Grid fill (or the decoded JData volume), detectors masked.  Gives
 * the bytes of umcx_job_labels.  Works for jobs parsed with or without UMCX_JOB_DEVICE_LABELS. */
int umcx_job_build_labels(const umcx_job* job, umcx_context* ctx, uint8_t* d_labels);

/* The rasterised domain with the reference's int32 encoding (sign bit = detector voxel), for --dumpmask parity
 * (UMCX_ERR_INPUT for a job parsed with UMCX_JOB_DEVICE_LABELS, whose domain exists only on the device). */
int umcx_job_domain_dims(const umcx_job* job, uint32_t dims[3]);
int umcx_job_domain_int32(const umcx_job* job, int32_t* out, size_t n);
/* Write <ID>_vol.bnii like --dumpmask (L528-531) to `path`. */
int umcx_job_dump_mask(const umcx_job* job, const char* path);
/* Write <ID>.bnii and <ID>_detp.jdb in the current directory like L841-842 (normalize != 0 applies). */
int umcx_job_write_outputs(const umcx_job* job, const float* fluence, const float* detp, const umcx_result* res,
                           int normalize);

/* The reference's main() (L868-875): runs a command line, prints "umcx encounters an error:" and returns 1 on
 * failure. */
int umcx_main(int argc, char* argv[]);

#ifdef __cplusplus
}
#endif

#endif /* UMCX_HOST_H */
