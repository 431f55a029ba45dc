// Internal interfaces between the host engine (mq_engine.cpp) and the CUDA translation
// units.  Not part of the public ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "mq_phys.h"

namespace mqd {

struct DevGrid {
    const float4* rf;   // RF E per volt, w = conductor mask
    const float4* ac;   // AC E per volt
    const float4* dc;   // combined static DC
    int32_t nx, ny, nz, pad;
    double h;
    double inv_h;       // 1 / h, correctly rounded (the FP64 kernel's division by h)
};

struct DevIons {        // device structure of arrays (FP64 state)
    double *x, *y, *z, *vx, *vy, *vz, *ph_rf, *ph_ac;
    uint64_t* rng;
    uint32_t *steps, *ncoll;
    int32_t *leg, *status;
    uint32_t* jid;
};

struct JobTable {       // per-job device data for injection
    const mqp::JobC* jc;
    const uint64_t* first;   // first ion index of each job (njobs + 1 entries)
    const uint64_t* seed;
    uint32_t njobs;
};

// per-job counters written by the summary kernel: [crashed, returned, transmitted, left, timeout, n, sum_coll, sum_steps]
constexpr int kCounters = 8;

// ---- mq_f64.cu
cudaError_t launch_inject(const mqp::Batch& b, JobTable jt, DevIons io, uint32_t n, cudaStream_t s);
cudaError_t launch_f64_step(DevGrid g, const mqp::Batch& b, const mqp::JobC* jc, const double2* rf_tab,
                            const double2* ac_tab, uint32_t tlen, DevIons io, uint32_t n, uint32_t max_more,
                            unsigned long long* d_steps, uint32_t* d_live, cudaStream_t s);
cudaError_t launch_phase_table(double w, uint32_t len, double2* out, cudaStream_t s);
cudaError_t launch_dc_combine(const float4* b0, const float4* b1, const float4* b2, const float4* b3,
                              float v0, float v1, float v2, float v3, float4* out, size_t n, cudaStream_t s);
cudaError_t launch_summarize(DevIons io, uint32_t n, uint32_t njobs, unsigned long long* counters, cudaStream_t s);

}  // namespace mqd

struct mq_physics;
struct mq_rfac;
struct mq_job;
namespace mqd {
// ---- mq_engine.cpp: the engine's batch / job constants for other translation units
mqp::Batch host_batch(int32_t nx, int32_t ny, int32_t nz, double h, double axis_mm, const double layers_mm[8],
                      const mq_physics& ph, const mq_rfac& rf);
mqp::JobC host_job(const mq_job& j, const mq_physics& ph);
// the checks every batch entry point applies to its jobs and physics, without an engine: a batch
// of at least one job sharing one RF drive, species with mass, z > 0 and ccs_n2 >= 0, physics with
// dt, temp_k > 0 and t_max, pressure_pa >= 0.  Returns MQ_OK or the status, with *why the reason.
int32_t check_jobs(const mq_job* jobs, size_t njobs, const mq_physics* ph, const char** why);

}  // namespace mqd
