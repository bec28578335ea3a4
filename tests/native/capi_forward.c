/* A plain-C caller of the library: parses a reference-style command line with the job API (umcx_host.h), runs the
 * forward simulation through umcx_gpu_forward (umcx_gpu.h) and prints the absorbed fraction and the detected-photon
 * count.  Built by the CPU tests (the headers must be valid C), run by the GPU tests. */
#include <stdio.h>
#include <stdlib.h>

#include "umcx_host.h"

int main(int argc, char** argv) {
    umcx_job* job = NULL;
    if (umcx_job_from_args(&job, argc, (const char* const*)argv) != UMCX_OK) {
        fprintf(stderr, "input error: %s\n", umcx_job_error(job));
        umcx_job_free(job);
        return 1;
    }
    const umcx_sim* s = umcx_job_sim(job);
    const size_t nout = (size_t)s->dim[0] * s->dim[1] * s->dim[2] * s->dim[3];
    const size_t ndet = s->issavedet ? (size_t)s->maxdetphotons * (size_t)umcx_detp_columns(s) : 1;
    float* fluence = (float*)malloc(nout * sizeof(float));
    float* detp = (float*)malloc(ndet * sizeof(float));
    umcx_context* ctx = NULL;
    int rc = umcx_create(&ctx, 0);
    if (rc != UMCX_OK) {
        fprintf(stderr, "no device (status %d)\n", rc);
        free(fluence);
        free(detp);
        umcx_job_free(job);
        return 2;
    }
    umcx_result r;
    rc = umcx_gpu_forward(ctx, s, umcx_job_labels(job), umcx_job_media(job), umcx_job_detpos(job), fluence, detp, &r);
    if (rc != UMCX_OK) {
        fprintf(stderr, "forward failed (status %d): %s\n", rc, umcx_last_error(ctx));
    } else {
        printf("absorbed %.6f detected %llu launched %llu kernel_ms %.3f\n",
               (r.energy_total - r.energy_escape) / r.energy_total, (unsigned long long)r.detected,
               (unsigned long long)r.launched, r.kernel_ms);
    }
    umcx_destroy(ctx);
    free(fluence);
    free(detp);
    umcx_job_free(job);
    return rc == UMCX_OK ? 0 : 3;
}
