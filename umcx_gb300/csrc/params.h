// params.h - host-side checks and derived constants of one simulation, shared by every entry point that launches
// the propagation kernels (capi.cu, noalloc.cu), so that their input rules and kernel parameters cannot drift apart.
//
// The fields follow MCX_param as filled by MCX_run_simulation (fangq/umcx src/umcx.cpp:787-796) and the optical table
// MCX_medium (L89-93, L800-806).
#pragma once

#include <cmath>
#include <cstring>

#include "../../include/umcx_gpu.h"
#include "propagate.cuh"

namespace umcx_dev {

// wall-clock budget of one propagation launch when umcx_tuning.budget_ms is 0 (5 minutes)
constexpr unsigned long long kDefaultBudgetNs = 300ULL * 1000000000ULL;

// nullptr when the simulation description is usable, else the reason it is rejected
inline const char* check_sim(const umcx_sim* s) {
    if (!s) return "sim is NULL";
    if (s->flags & ~UMCX_SIM_FLAGS_ALL) return "unknown bits in umcx_sim.flags";
    for (int k = 0; k < 3; k++)
        if (s->dim[k] < 1 || s->dim[k] > 32767) return "dim[0..2] must be in 1..32767";
    if (s->dim[3] < 1 || s->dim[3] > UMCX_MAX_GATES) return "dim[3] (time gates) must be in 1..65535";
    const unsigned long long nvox = 1ULL * s->dim[0] * s->dim[1] * s->dim[2];
    if (nvox * s->dim[3] >= (1ULL << 31)) return "voxels x gates must be below 2^31";
    if (s->mediumnum < 1 || s->mediumnum > UMCX_MAX_MEDIA) return "mediumnum must be in 1..128";
    if (s->detnum < 0 || s->detnum > UMCX_MAX_DET) return "detnum must be in 0..64";
    if (!(s->rtstep > 0.f) || !std::isfinite(s->rtstep) || !std::isfinite(s->tstart) || !std::isfinite(s->tend))
        return "invalid time window";
    if (s->srctype < 0 || s->srctype > 6) return "unknown source type";
    return nullptr;
}

// per-label constants of the kernels' shared-memory table (see Medium)
inline Medium make_medium(const float* m, int outputtype) {
    Medium r;
    const float mua = m[0], mus = m[1], g = m[2], n = m[3];
    r.a = make_float4(mua, mus, g, n);
    r.b = make_float4(mus != 0.f ? 1.f / mus : 0.f, deposit_factor(mua, outputtype), g != 0.f ? 1.f / (2.f * g) : 0.f,
                      n * kOneOverC0);
    r.c = make_float4(1.f - g * g, 1.f - g, 2.f * g, 1.f + g * g);
    return r;
}

// kernel parameters of a checked simulation description; detpos holds detnum {x, y, z, r} rows (NULL: no
// detector table, for callers that stage detectors elsewhere)
inline KParams make_params(const umcx_sim* s, const float* detpos) {
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
    P.gate_off = -(s->tstart * s->rtstep);
    P.unitinmm = s->unitinmm;
    P.isreflect = s->isreflect;
    P.issavevol = s->issavevol;
    P.issavedet = s->issavedet;
    // a simulation that saves no records has no record fields: the kernels that keep partial paths for several
    // simulations at once (the batch) test only savedetflag, and size the per-lane slots by ppathlen
    P.savedetflag = s->issavedet ? s->savedetflag : 0;
    P.mediumnum = s->mediumnum;
    P.outputtype = s->outputtype;
    P.detnum = s->detnum;
    P.srctype = s->srctype;
    P.maxdetphotons = s->issavedet ? s->maxdetphotons : 0u;
    P.cols = umcx_detp_columns(s);
    P.ppathlen = (s->issavedet && (s->savedetflag & UMCX_DET_PPATH)) ? s->mediumnum : 0;
    for (int k = 0; k < 4; k++) P.seeds[k] = s->seeds[k];
    P.srcpos = make_float4(s->srcpos[0], s->srcpos[1], s->srcpos[2], 1.f);
    P.srcdir = make_float4(s->srcdir[0], s->srcdir[1], s->srcdir[2], 0.f);
    P.srcrdir = make_float4(1.f / s->srcdir[0], 1.f / s->srcdir[1], 1.f / s->srcdir[2], 0.f);
    P.srcparam1 = make_float4(s->srcparam1[0], s->srcparam1[1], s->srcparam1[2], s->srcparam1[3]);
    P.srcparam2 = make_float4(s->srcparam2[0], s->srcparam2[1], s->srcparam2[2], s->srcparam2[3]);
    P.budget_ns = kDefaultBudgetNs;
    for (int d = 0; detpos && d < s->detnum; d++)
        P.det[d] = make_float4(detpos[4 * d], detpos[4 * d + 1], detpos[4 * d + 2], detpos[4 * d + 3]);
    return P;
}

}  // namespace umcx_dev
