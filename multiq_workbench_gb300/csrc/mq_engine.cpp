// Host engine behind the C ABI (include/mq_engine.h): device field buffers, the combined
// DC cache, batch / job constants, injection, the launch loops of the FP64 and mixed
// kernels, and the per-job summary.
//
// Reference: chsim Engine (simulation/chsim/src/channel.rs:309-506) and its tiled launch
// loop (simulation/chsim/src/tiled.rs:87-218).  Unlike the reference, nothing here
// panics: every failure is an mq_status plus a message for mq_last_error.
#include "mq_engine.h"
#include "mq_internal.h"
#include "mq_mixed.h"

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

using mqp::Batch;
using mqp::JobC;

namespace {

struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
    cudaError_t grow(size_t bytes) {
        if (bytes <= cap) return cudaSuccess;
        if (p) { cudaFree(p); p = nullptr; cap = 0; }
        cudaError_t e = cudaMalloc(&p, bytes);
        if (e == cudaSuccess) cap = bytes;
        return e;
    }
    void release() { if (p) cudaFree(p); p = nullptr; cap = 0; }
    template <class T> T* as() const { return static_cast<T*>(p); }
};

// page-locked host staging area for the per-call job tables and counters (so the
// host<->device copies of a call are true asynchronous DMA); grown only between calls
struct HostBuf {
    void* p = nullptr;
    size_t cap = 0;
    cudaError_t grow(size_t bytes) {
        if (bytes <= cap) return cudaSuccess;
        if (p) { cudaFreeHost(p); p = nullptr; cap = 0; }
        cudaError_t e = cudaMallocHost(&p, bytes);
        if (e == cudaSuccess) cap = bytes;
        return e;
    }
    void release() { if (p) cudaFreeHost(p); p = nullptr; cap = 0; }
    char* at(size_t off) const { return static_cast<char*>(p) + off; }
};

constexpr uint32_t kTabCap = 1u << 20;        // phase-table length cap (longer runs evaluate directly)
constexpr uint32_t kF64Chunk = 50000;         // steps per FP64 launch

}  // namespace

struct mq_engine {
    int dev = 0;
    int prec = MQ_PREC_F64;
    std::string err;
    int32_t nx = 0, ny = 0, nz = 0;
    double h = 0, axis_mm = 0, layers[8] = {0};
    size_t nnodes = 0;
    float4 *d_rf = nullptr, *d_ac = nullptr, *d_dc = nullptr;
    float4* d_dcb[4] = {nullptr, nullptr, nullptr, nullptr};
    double dc_cur[4] = {0, 0, 0, 0};
    bool dc_valid = false;
    uint64_t grid_gen = 0;         // bumped whenever the combined DC field changes
    cudaStream_t st = nullptr;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    DevBuf ions[14];
    DevBuf jobc, jfirst, jseed, tabs, counters, misc;
    HostBuf stage;                 // pinned staging: [job constants | job offsets | job seeds | counters]
    mqmix::Scratch mix;            // mixed-engine scratch (lists, queue counters, job table)
    mqmix::Tuning tune;            // launch shape of the mixed engine
    int32_t fault = MQ_FAULT_NONE; // one-shot host-side fault for the next stepping call
};

namespace {

mq_status fail(mq_engine* e, mq_status code, const std::string& msg) {
    if (e) e->err = msg;
    return code;
}
mq_status cuda_fail(mq_engine* e, cudaError_t c, const char* what) {
    cudaGetLastError();   // clear a non-sticky error (failed allocation, bad launch shape) so later calls start clean
    std::string m = std::string(what) + ": " + cudaGetErrorString(c);
    return fail(e, c == cudaErrorMemoryAllocation ? MQ_ERR_NOMEM : MQ_ERR_CUDA, m);
}
#define CK(call, what) do { cudaError_t c_ = (call); if (c_ != cudaSuccess) return cuda_fail(e, c_, what); } while (0)

// legacy_mfp_mean (channel.rs:376-381)
double legacy_mfp_mean(const mq_job& j, const mq_physics& ph) {
    double p_torr = ph.pressure_pa / 133.322 + 1e-10;
    double np = 2.68e5 * (p_torr / 760.0);
    double m = j.sp.mass;
    double ccs_he = 2.81e-9 * m * m * m - 3.55e-5 * m * m + 0.232 * m + 41.91;
    double ccs = ccs_he * 10.0 * sqrt(j.sp.z);
    return 1.0 / (np * ccs);
}

uint32_t max_steps_of(const mq_physics& ph) {
    double s = floor(ph.t_max / ph.dt + 0.5);   // (T_MAX / DT).round(), world.rs:360
    if (!(s >= 0)) return 0;
    if (s > 4294967295.0) return 4294967295u;
    return (uint32_t)s;
}

// batch_params (channel.rs:397-410) in f64
Batch make_batch(const mq_engine* e, const mq_physics& ph, const mq_rfac& rf) {
    Batch b;
    std::memset(&b, 0, sizeof(b));
    b.dt = ph.dt;
    b.v_rf = rf.v_rf;
    b.w_rf = rf.f_rf * ph.dt;
    b.h = e->h;
    if (ph.legacy_criteria) {
        b.z_return = 1.0e-3;
        b.z_exit = 23.7e-3;
        b.crash_z0 = e->layers[0] * 1e-3;
        b.crash_z1 = e->layers[1] * 1e-3;
    } else {
        b.z_return = 0.5e-3;
        b.z_exit = e->layers[4] * 1e-3;
        b.crash_z0 = -1.0;
        b.crash_z1 = 1.0;
    }
    b.lim[0] = (double)(e->nx - 1) * e->h;
    b.lim[1] = (double)(e->ny - 1) * e->h;
    b.lim[2] = (double)(e->nz - 1) * e->h;
    b.a = e->axis_mm * 1e-3;
    b.z_inject = ph.z_inject_mm * 1e-3;
    b.r_inject = ph.r_inject_mm * 1e-3;
    b.sigma = ph.sigma_mm * 1e-3;
    b.nx = e->nx; b.ny = e->ny; b.nz = e->nz;
    b.max_steps = max_steps_of(ph);
    b.nearest = ph.legacy_fields ? 1 : 0;
    b.legacy_coll = ph.legacy_collisions ? 1 : 0;
    b.launch = ph.legacy_injection ? MQ_LAUNCH_LEGACY : ph.launch;
    b.rf_phase0 = ph.rf_phase0 ? 1 : 0;
    return b;
}

// job_params (channel.rs:412-426) in f64
JobC make_job(const mq_job& j, const mq_physics& ph) {
    JobC c;
    std::memset(&c, 0, sizeof(c));
    double m = j.sp.mass * mqp::AMU, mg = 28.0 * mqp::AMU;
    double qm = j.sp.z * mqp::QE / m;
    double n_gas = ph.pressure_pa / (mqp::KB * ph.temp_k);
    double s_gas = sqrt(mqp::KB * ph.temp_k / mg);
    double qk = ph.legacy_force ? 0.5 * qm : qm;
    c.qmdt = qk * ph.dt;
    c.v_ac = j.drive.v_ac;
    c.w_ac = j.drive.f_ac * ph.dt;
    c.nsd = (n_gas * (j.sp.ccs_n2 * 1e-20)) * ph.dt;
    c.s_gas = s_gas;
    c.mr = mg / (m + mg);
    c.floor_v = ph.legacy_collisions ? sqrt(2.0 * 0.035 * 1.6e-19 / (j.sp.mass * 1.66e-27)) : -1.0;
    c.mfp_mean = legacy_mfp_mean(j, ph);
    c.s_ion = sqrt(mqp::KB * ph.temp_k / m);
    c.m = m;
    c.zc = j.sp.z;
    c.use_ac = j.drive.v_ac != 0.0 ? 1 : 0;
    c.tab = 0;
    return c;
}

mq_status check_batch(mq_engine* e, const mq_job* jobs, size_t njobs, const mq_physics* ph) {
    if (!e) return MQ_ERR_INVALID;
    const char* why = nullptr;
    const mq_status s = mqd::check_jobs(jobs, njobs, ph, &why);
    return s == MQ_OK ? MQ_OK : fail(e, s, why);
}

mqd::DevIons dev_ions(mq_engine* e) {
    mqd::DevIons d;
    d.x = e->ions[0].as<double>(); d.y = e->ions[1].as<double>(); d.z = e->ions[2].as<double>();
    d.vx = e->ions[3].as<double>(); d.vy = e->ions[4].as<double>(); d.vz = e->ions[5].as<double>();
    d.ph_rf = e->ions[6].as<double>(); d.ph_ac = e->ions[7].as<double>();
    d.rng = e->ions[8].as<uint64_t>();
    d.steps = e->ions[9].as<uint32_t>(); d.ncoll = e->ions[10].as<uint32_t>();
    d.leg = e->ions[11].as<int32_t>(); d.status = e->ions[12].as<int32_t>(); d.jid = e->ions[13].as<uint32_t>();
    return d;
}

const size_t kIonBytes[14] = {8, 8, 8, 8, 8, 8, 8, 8, 8, 4, 4, 4, 4, 4};

void* host_field(const mq_ions* io, int k) {
    switch (k) {
        case 0: return io->x; case 1: return io->y; case 2: return io->z;
        case 3: return io->vx; case 4: return io->vy; case 5: return io->vz;
        case 6: return io->ph_rf; case 7: return io->ph_ac; case 8: return io->rng;
        case 9: return io->steps; case 10: return io->ncoll; case 11: return io->leg;
        case 12: return io->status; default: return io->jid;
    }
}

mq_status grow_ions(mq_engine* e, size_t n) {
    for (int k = 0; k < 14; ++k) CK(e->ions[k].grow(kIonBytes[k] * (n ? n : 1)), "device ion buffers");
    return MQ_OK;
}

mq_status copy_ions(mq_engine* e, const mq_ions* io, size_t n, bool to_device, uint64_t* bytes) {
    for (int k = 0; k < 14; ++k) {
        void* hp = host_field(io, k);
        if (!hp) return fail(e, MQ_ERR_INVALID, "ion state array missing");
        size_t b = kIonBytes[k] * n;
        if (to_device) CK(cudaMemcpyAsync(e->ions[k].p, hp, b, cudaMemcpyHostToDevice, e->st), "ion upload");
        else CK(cudaMemcpyAsync(hp, e->ions[k].p, b, cudaMemcpyDeviceToHost, e->st), "ion download");
        if (bytes) *bytes += b;
    }
    return MQ_OK;
}

// layout of the pinned staging area for a call with njobs jobs
struct StageLayout {
    size_t jc, first, seed, cnt, total;
    explicit StageLayout(size_t njobs) {
        auto up = [](size_t v) { return (v + 255) & ~size_t(255); };
        jc = 0;
        first = up(sizeof(JobC) * njobs);
        seed = first + up(8 * (njobs + 1));
        cnt = seed + up(8 * njobs);
        total = cnt + up(sizeof(unsigned long long) * mqd::kCounters * njobs);
    }
};

// job constants (and, for device injection, job offsets and seeds) staged in pinned memory
// and uploaded; phase tables for the FP64 kernel; returns the table length
mq_status upload_jobs(mq_engine* e, const mq_job* jobs, size_t njobs, const mq_physics& ph, const Batch& b,
                      bool offsets, uint32_t* tlen_out, size_t* ntab_out, uint64_t* h2d) {
    const StageLayout L(njobs);
    CK(e->stage.grow(L.total), "pinned staging");
    JobC* jc = reinterpret_cast<JobC*>(e->stage.at(L.jc));
    std::vector<double> tones;
    for (size_t k = 0; k < njobs; ++k) {
        jc[k] = make_job(jobs[k], ph);
        size_t t = 0;
        for (; t < tones.size(); ++t) if (tones[t] == jc[k].w_ac) break;
        if (t == tones.size()) tones.push_back(jc[k].w_ac);
        jc[k].tab = (int32_t)t;
    }
    uint32_t tlen = b.max_steps < kTabCap ? b.max_steps : kTabCap;
    if (tlen == 0) tlen = 1;
    CK(e->jobc.grow(sizeof(JobC) * njobs), "job table");
    CK(cudaMemcpyAsync(e->jobc.p, jc, sizeof(JobC) * njobs, cudaMemcpyHostToDevice, e->st), "job table upload");
    *h2d += sizeof(JobC) * njobs;
    if (offsets) {
        uint64_t* first = reinterpret_cast<uint64_t*>(e->stage.at(L.first));
        uint64_t* seed = reinterpret_cast<uint64_t*>(e->stage.at(L.seed));
        first[0] = 0;
        for (size_t k = 0; k < njobs; ++k) { first[k + 1] = first[k] + jobs[k].n; seed[k] = jobs[k].seed; }
        CK(e->jfirst.grow(8 * (njobs + 1)), "job offsets");
        CK(e->jseed.grow(8 * njobs), "job seeds");
        CK(cudaMemcpyAsync(e->jfirst.p, first, 8 * (njobs + 1), cudaMemcpyHostToDevice, e->st), "job upload");
        CK(cudaMemcpyAsync(e->jseed.p, seed, 8 * njobs, cudaMemcpyHostToDevice, e->st), "job upload");
        *h2d += 8 * (2 * njobs + 1);
    }
    if (e->prec == MQ_PREC_MIXED) {   // the mixed engine advances its phases itself: no tables
        *tlen_out = 0;
        *ntab_out = 0;
        return MQ_OK;
    }
    size_t ntab = 1 + tones.size();
    CK(e->tabs.grow(sizeof(double2) * (size_t)tlen * ntab), "phase tables");
    double2* t0 = e->tabs.as<double2>();
    CK(mqd::launch_phase_table(b.w_rf, tlen, t0, e->st), "phase table kernel");
    for (size_t t = 0; t < tones.size(); ++t)
        CK(mqd::launch_phase_table(tones[t], tlen, t0 + (size_t)tlen * (1 + t), e->st), "phase table kernel");
    *tlen_out = tlen;
    *ntab_out = ntab;
    return MQ_OK;
}

mqd::DevGrid dev_grid(const mq_engine* e) {
    mqd::DevGrid g;
    g.rf = e->d_rf; g.ac = e->d_ac; g.dc = e->d_dc;
    g.nx = e->nx; g.ny = e->ny; g.nz = e->nz; g.pad = 0; g.h = e->h; g.inv_h = 1.0 / e->h;
    return g;
}

// FP64 launch loop (chsim run_direct, channel.rs:478-493): relaunch until no ion is live
// or the step budget is spent.  Each launch advances every live ion by <= kF64Chunk steps.
mq_status run_f64(mq_engine* e, const Batch& b, uint32_t tlen, size_t n, uint32_t max_more, mq_run_stats* stats,
                  uint64_t* steps_out) {
    const int32_t fault = e->fault;
    e->fault = MQ_FAULT_NONE;
    if (fault == MQ_FAULT_ALLOC) return fail(e, MQ_ERR_NOMEM, "FP64 engine: injected device allocation failure");
    if (fault == MQ_FAULT_LAUNCH) return fail(e, MQ_ERR_CUDA, "FP64 engine: injected kernel launch failure");
    // every ion times out at max_steps, so ceil(min(max_more, max_steps) / chunk) launches finish
    // every ion; one more is allowed before the watchdog calls it
    const uint64_t need = max_more < b.max_steps ? (uint64_t)max_more : (uint64_t)b.max_steps;
    const uint64_t max_launches = fault == MQ_FAULT_LAUNCH_BUDGET ? 1 : (need + kF64Chunk - 1) / kF64Chunk + 1;
    const uint32_t chunk = fault == MQ_FAULT_LAUNCH_BUDGET ? 16u : kF64Chunk;
    CK(e->misc.grow(64), "counters");
    unsigned long long* d_steps = e->misc.as<unsigned long long>();
    uint32_t* d_live = reinterpret_cast<uint32_t*>(d_steps + 1);
    CK(cudaMemsetAsync(d_steps, 0, 16, e->st), "counter reset");
    const double2* rf_tab = e->tabs.as<double2>();
    const double2* ac_tab = rf_tab + tlen;
    uint64_t budget = max_more;
    uint32_t launches = 0, live = 0;
    float step_ms = 0.0f;
    for (;;) {
        uint32_t L = budget < chunk ? (uint32_t)budget : chunk;
        if (L == 0 || launches >= max_launches) break;
        CK(cudaMemsetAsync(d_live, 0, 4, e->st), "counter reset");
        CK(cudaEventRecord(e->ev[2], e->st), "event");
        CK(mqd::launch_f64_step(dev_grid(e), b, e->jobc.as<JobC>(), rf_tab, ac_tab, tlen, dev_ions(e), (uint32_t)n, L,
                                d_steps, d_live, e->st), "FP64 step kernel");
        CK(cudaEventRecord(e->ev[3], e->st), "event");
        live = 0;
        CK(cudaMemcpyAsync(&live, d_live, 4, cudaMemcpyDeviceToHost, e->st), "live count");
        CK(cudaStreamSynchronize(e->st), "FP64 step kernel");
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e->ev[2], e->ev[3]);
        step_ms += ms;
        ++launches;
        budget -= L;
        if (live == 0) break;
    }
    unsigned long long steps = 0;
    CK(cudaMemcpyAsync(&steps, d_steps, 8, cudaMemcpyDeviceToHost, e->st), "step count");
    CK(cudaStreamSynchronize(e->st), "step count");
    *steps_out = steps;
    if (stats) {
        stats->launches += launches;
        stats->kernel_launches += launches;
        stats->step_kernel_launches += launches;
        stats->step_kernel_ms += step_ms;
    }
    if (live != 0 && max_more >= b.max_steps)
        return fail(e, MQ_ERR_WATCHDOG, "FP64 engine: launch budget exhausted with " + std::to_string(live) + " live ions");
    return MQ_OK;
}

mq_status run_mixed(mq_engine* e, const mq_job* jobs, size_t njobs, const mq_physics& ph, const Batch& b, size_t n,
                    uint32_t max_more, int write_states, mq_run_stats* stats, uint64_t* steps_out) {
    std::vector<mqmix::MixJob> mj(njobs);
    for (size_t k = 0; k < njobs; ++k) mj[k] = mqmix::make_mix_job(make_job(jobs[k], ph), b);
    const int32_t fault = e->fault;
    e->fault = MQ_FAULT_NONE;
    if (fault == MQ_FAULT_ALLOC) return fail(e, MQ_ERR_NOMEM, "mixed engine: injected device allocation failure");
    if (fault == MQ_FAULT_LAUNCH) return fail(e, MQ_ERR_CUDA, "mixed engine: injected kernel launch failure");
    mqmix::Tuning tune = e->tune;
    if (fault == MQ_FAULT_LAUNCH_BUDGET) {   // one launch of 16 steps
        tune.max_launches = 1;
        tune.chunk = 16;
    }
    mqmix::RunInfo info;
    cudaError_t c = mqmix::run(e->mix, tune, dev_grid(e), e->grid_gen, b, mj.data(), njobs, dev_ions(e), (uint32_t)n,
                               max_more, write_states, e->st, &info);
    if (c != cudaSuccess) return cuda_fail(e, c, "mixed engine");
    *steps_out = info.ion_steps;
    if (info.watchdog)
        return fail(e, MQ_ERR_WATCHDOG, "mixed engine: launch budget exhausted with " + std::to_string(info.survivors) +
                                            " live ions");
    if (stats) {
        stats->launches += info.graph_replays;
        stats->graph_replays += info.graph_replays;
        stats->cell_loads += info.cell_loads;
        stats->ions_queued += info.ions_queued;
        stats->kernel_launches += info.kernel_launches;
        stats->step_kernel_launches += info.step_launches;
        stats->step_kernel_ms += info.step_ms;
    }
    return MQ_OK;
}

}  // namespace

// batch and job constants for code outside this file (same functions the engine uses)
namespace mqd {
Batch host_batch(int32_t nx, int32_t ny, int32_t nz, double h, double axis_mm, const double layers_mm[8],
                 const mq_physics& ph, const mq_rfac& rf) {
    mq_engine tmp;   // geometry only
    tmp.nx = nx; tmp.ny = ny; tmp.nz = nz; tmp.h = h; tmp.axis_mm = axis_mm;
    for (int i = 0; i < 8; ++i) tmp.layers[i] = layers_mm[i];
    return make_batch(&tmp, ph, rf);
}
JobC host_job(const mq_job& j, const mq_physics& ph) { return make_job(j, ph); }

mq_status check_jobs(const mq_job* jobs, size_t njobs, const mq_physics* ph, const char** why) {
    *why = nullptr;
    if (!jobs || njobs == 0) { *why = "a batch needs at least one job"; return MQ_ERR_INVALID; }   // channel.rs:444
    if (!ph || !(ph->dt > 0) || !(ph->t_max >= 0) || !(ph->temp_k > 0) || !(ph->pressure_pa >= 0)) {
        *why = "physics: dt, temp_k must be > 0 and t_max, pressure_pa >= 0";
        return MQ_ERR_INVALID;
    }
    for (size_t k = 0; k < njobs; ++k) {
        if (jobs[k].drive.v_rf != jobs[0].drive.v_rf || jobs[k].drive.f_rf != jobs[0].drive.f_rf) {
            *why = "RF drive must be shared by a batch";   // channel.rs:446
            return MQ_ERR_RF_MISMATCH;
        }
        if (!(jobs[k].sp.mass > 0) || !(jobs[k].sp.z > 0) || !(jobs[k].sp.ccs_n2 >= 0)) {
            *why = "species: mass and z must be > 0, ccs_n2 >= 0";
            return MQ_ERR_INVALID;
        }
    }
    return MQ_OK;
}
}  // namespace mqd

extern "C" {

int32_t mq_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) { cudaGetLastError(); return 0; }
    return n;
}

mq_status mq_engine_create(const mq_grid_desc* g, int32_t precision, int32_t device, mq_engine** out) {
    if (!out) return MQ_ERR_INVALID;
    *out = nullptr;
    if (!g || !g->rf4 || !g->ac4 || g->nx < 3 || g->ny < 3 || g->nz < 3 || !(g->h > 0)) return MQ_ERR_INVALID;
    if (precision != MQ_PREC_F64 && precision != MQ_PREC_MIXED) return MQ_ERR_INVALID;
    if (mq_device_count() <= device || device < 0) return MQ_ERR_NO_DEVICE;   // expect("no Metal device"), channel.rs:328
    mq_engine* e = new (std::nothrow) mq_engine();
    if (!e) return MQ_ERR_NOMEM;
    e->dev = device;
    e->prec = precision;
    e->nx = g->nx; e->ny = g->ny; e->nz = g->nz; e->h = g->h; e->axis_mm = g->axis_mm;
    for (int i = 0; i < 8; ++i) e->layers[i] = g->layers_mm[i];
    e->nnodes = (size_t)g->nx * g->ny * g->nz;
    auto bail = [&](mq_status s) { mq_engine_destroy(e); return s; };
    // the mixed kernel addresses its 3 (or 4, wide) float4 of node record per node with 32-bit offsets
    if (precision == MQ_PREC_MIXED && 3 * e->nnodes >= ((size_t)1 << 32)) {
        e->err = "grid too large for the mixed engine (3 x nodes must be below 2^32)";
        return bail(MQ_ERR_TOO_LARGE);
    }
    if (cudaSetDevice(device) != cudaSuccess) return bail(MQ_ERR_CUDA);
    if (cudaStreamCreateWithFlags(&e->st, cudaStreamNonBlocking) != cudaSuccess) return bail(MQ_ERR_CUDA);
    for (auto& v : e->ev) if (cudaEventCreate(&v) != cudaSuccess) return bail(MQ_ERR_CUDA);
    const size_t bytes = e->nnodes * sizeof(float4);
    float4** dst[6] = {&e->d_rf, &e->d_ac, &e->d_dcb[0], &e->d_dcb[1], &e->d_dcb[2], &e->d_dcb[3]};
    const float* src[6] = {g->rf4, g->ac4, g->dc4[0], g->dc4[1], g->dc4[2], g->dc4[3]};
    for (int k = 0; k < 6; ++k) {
        if (!src[k]) continue;
        if (cudaMalloc((void**)dst[k], bytes) != cudaSuccess) { cudaGetLastError(); return bail(MQ_ERR_NOMEM); }
        if (cudaMemcpy(*dst[k], src[k], bytes, cudaMemcpyHostToDevice) != cudaSuccess) return bail(MQ_ERR_CUDA);
    }
    if (cudaMalloc((void**)&e->d_dc, bytes) != cudaSuccess) { cudaGetLastError(); return bail(MQ_ERR_NOMEM); }
    if (cudaMemset(e->d_dc, 0, bytes) != cudaSuccess) return bail(MQ_ERR_CUDA);
    e->tune = mqmix::default_tuning(device, e->nnodes);
    *out = e;
    return MQ_OK;
}

void mq_engine_destroy(mq_engine* e) {
    if (!e) return;
    cudaSetDevice(e->dev);
    if (e->st) cudaStreamSynchronize(e->st);
    for (float4* p : {e->d_rf, e->d_ac, e->d_dc, e->d_dcb[0], e->d_dcb[1], e->d_dcb[2], e->d_dcb[3]}) if (p) cudaFree(p);
    for (auto& b : e->ions) b.release();
    e->jobc.release(); e->jfirst.release(); e->jseed.release(); e->tabs.release(); e->counters.release(); e->misc.release();
    e->stage.release();
    mqmix::release(e->mix);
    for (auto& v : e->ev) if (v) cudaEventDestroy(v);
    if (e->st) cudaStreamDestroy(e->st);
    delete e;
}

const char* mq_last_error(mq_engine* e) { return e ? e->err.c_str() : "null engine"; }

mq_status mq_engine_set_dc(mq_engine* e, const double dc[4]) {
    if (!e || !dc) return MQ_ERR_INVALID;
    if (e->dc_valid && std::memcmp(dc, e->dc_cur, sizeof(e->dc_cur)) == 0) return MQ_OK;   // dc cache hit
    CK(cudaSetDevice(e->dev), "cudaSetDevice");
    CK(mqd::launch_dc_combine(e->d_dcb[0], e->d_dcb[1], e->d_dcb[2], e->d_dcb[3], (float)dc[0], (float)dc[1],
                              (float)dc[2], (float)dc[3], e->d_dc, e->nnodes, e->st), "DC combine kernel");
    CK(cudaStreamSynchronize(e->st), "DC combine kernel");
    std::memcpy(e->dc_cur, dc, sizeof(e->dc_cur));
    e->dc_valid = true;
    e->grid_gen += 1;
    return MQ_OK;
}

static mq_status inject_host(mq_engine* e, const mq_job* jobs, size_t njobs, const mq_physics* ph, mq_ions* out, size_t n) {
    mq_status s = check_batch(e, jobs, njobs, ph);
    if (s != MQ_OK) return s;
    if (!out) return fail(e, MQ_ERR_INVALID, "no output states");
    size_t tot = 0;
    for (size_t k = 0; k < njobs; ++k) tot += jobs[k].n;
    if (tot != n) return fail(e, MQ_ERR_INVALID, "n must equal the sum of the jobs' ion counts");
    Batch b = make_batch(e, *ph, jobs[0].drive);
    size_t i = 0;
    for (size_t k = 0; k < njobs; ++k) {
        JobC jc = make_job(jobs[k], *ph);
        for (uint64_t q = 0; q < jobs[k].n; ++q, ++i) {
            mqp::Ion0 o;
            mqp::inject_one(b, jc, mqp::splitmix(jobs[k].seed + q * 0x9E37ull), &o);
            out->x[i] = o.x[0]; out->y[i] = o.x[1]; out->z[i] = o.x[2];
            out->vx[i] = o.v[0]; out->vy[i] = o.v[1]; out->vz[i] = o.v[2];
            out->ph_rf[i] = o.ph_rf; out->ph_ac[i] = o.ph_ac; out->rng[i] = o.rng; out->leg[i] = o.leg;
            out->steps[i] = 0; out->ncoll[i] = 0; out->status[i] = 0; out->jid[i] = (uint32_t)k;
        }
    }
    return MQ_OK;
}

mq_status mq_inject(mq_engine* e, const mq_job* jobs, size_t njobs, const mq_physics* ph, mq_ions* out, size_t n) {
    return inject_host(e, jobs, njobs, ph, out, n);
}

mq_status mq_inject_grid(const mq_grid_desc* g, const mq_job* jobs, size_t njobs, const mq_physics* ph, mq_ions* out,
                         size_t n) {
    if (!g || g->nx < 3 || g->ny < 3 || g->nz < 3 || !(g->h > 0)) return MQ_ERR_INVALID;
    mq_engine tmp;   // geometry only; no device resources
    tmp.nx = g->nx; tmp.ny = g->ny; tmp.nz = g->nz; tmp.h = g->h; tmp.axis_mm = g->axis_mm;
    for (int i = 0; i < 8; ++i) tmp.layers[i] = g->layers_mm[i];
    return inject_host(&tmp, jobs, njobs, ph, out, n);
}

mq_status mq_run_ions(mq_engine* e, const mq_job* jobs, size_t njobs, const mq_physics* ph, mq_ions* io, size_t n,
                      uint32_t max_more, mq_run_stats* stats) {
    mq_status s = check_batch(e, jobs, njobs, ph);
    if (s != MQ_OK) return s;
    if (!io) return fail(e, MQ_ERR_INVALID, "no ion states");
    if (n > 0xFFFFFFF0ull) return fail(e, MQ_ERR_TOO_LARGE, "at most 2^32-16 ions per call");
    if (stats) std::memset(stats, 0, sizeof(*stats));
    if (!e->dc_valid) return fail(e, MQ_ERR_INVALID, "set the DC field first (mq_engine_set_dc)");
    CK(cudaSetDevice(e->dev), "cudaSetDevice");
    for (size_t i = 0; i < n; ++i)
        if (io->jid[i] >= njobs) return fail(e, MQ_ERR_INVALID, "ion job index out of range");
    Batch b = make_batch(e, *ph, jobs[0].drive);
    if ((s = grow_ions(e, n)) != MQ_OK) return s;
    uint64_t h2d = 0, d2h = 0;
    CK(cudaEventRecord(e->ev[0], e->st), "event");
    if ((s = copy_ions(e, io, n, true, &h2d)) != MQ_OK) return s;
    uint32_t tlen = 0;
    size_t ntab = 0;
    if ((s = upload_jobs(e, jobs, njobs, *ph, b, false, &tlen, &ntab, &h2d)) != MQ_OK) return s;
    uint64_t steps = 0;
    if (e->prec == MQ_PREC_F64) s = run_f64(e, b, tlen, n, max_more, stats, &steps);
    else s = run_mixed(e, jobs, njobs, *ph, b, n, max_more, 1, stats, &steps);
    if (s == MQ_ERR_WATCHDOG) {   // the states are the checkpoint: hand them back so the caller can resume
        const std::string why = e->err;
        mq_status s2 = copy_ions(e, io, n, false, &d2h);
        if (s2 == MQ_OK && cudaStreamSynchronize(e->st) != cudaSuccess) s2 = MQ_ERR_CUDA;
        if (s2 != MQ_OK) return s2;
        e->err = why;
        return s;
    }
    if (s != MQ_OK) return s;
    if ((s = copy_ions(e, io, n, false, &d2h)) != MQ_OK) return s;
    CK(cudaEventRecord(e->ev[1], e->st), "event");
    CK(cudaStreamSynchronize(e->st), "ion download");
    if (stats) {
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e->ev[0], e->ev[1]);
        stats->kernel_ms = ms;
        stats->ion_steps = steps;
        stats->h2d_bytes = h2d;
        stats->d2h_bytes = d2h;
        stats->kernel_launches += (uint32_t)ntab;
    }
    return MQ_OK;
}

mq_status mq_run_batch(mq_engine* e, const mq_job* jobs, size_t njobs, const double dc[4], const mq_physics* ph,
                       mq_outcome* out, mq_ions* ions_out, mq_run_stats* stats) {
    mq_status s = check_batch(e, jobs, njobs, ph);
    if (s != MQ_OK) return s;
    if (!out || !dc) return fail(e, MQ_ERR_INVALID, "outcome array and DC voltages are required");
    if (stats) std::memset(stats, 0, sizeof(*stats));
    size_t n = 0;
    for (size_t k = 0; k < njobs; ++k) n += jobs[k].n;
    if (n > 0xFFFFFFF0ull) return fail(e, MQ_ERR_TOO_LARGE, "at most 2^32-16 ions per batch");
    if ((s = mq_engine_set_dc(e, dc)) != MQ_OK) return s;
    CK(cudaSetDevice(e->dev), "cudaSetDevice");
    Batch b = make_batch(e, *ph, jobs[0].drive);
    if ((s = grow_ions(e, n)) != MQ_OK) return s;
    uint64_t h2d = 0, d2h = 0;
    CK(cudaEventRecord(e->ev[0], e->st), "event");
    uint32_t tlen = 0;
    size_t ntab = 0;
    if ((s = upload_jobs(e, jobs, njobs, *ph, b, true, &tlen, &ntab, &h2d)) != MQ_OK) return s;
    mqd::JobTable jt;
    jt.jc = e->jobc.as<JobC>(); jt.first = e->jfirst.as<uint64_t>(); jt.seed = e->jseed.as<uint64_t>(); jt.njobs = (uint32_t)njobs;
    if (e->prec == MQ_PREC_F64) CK(mqd::launch_inject(b, jt, dev_ions(e), (uint32_t)n, e->st), "inject kernel");
    else CK(mqmix::launch_inject(b, jt, dev_ions(e), (uint32_t)n, e->st), "inject kernel");
    uint64_t steps = 0;
    if (e->prec == MQ_PREC_F64) s = run_f64(e, b, tlen, n, 0xFFFFFFFFu, stats, &steps);
    else s = run_mixed(e, jobs, njobs, *ph, b, n, 0xFFFFFFFFu, ions_out ? 1 : 0, stats, &steps);
    if (s != MQ_OK) return s;
    CK(e->counters.grow(sizeof(unsigned long long) * mqd::kCounters * njobs), "job counters");
    CK(cudaMemsetAsync(e->counters.p, 0, sizeof(unsigned long long) * mqd::kCounters * njobs, e->st), "counter reset");
    CK(mqd::launch_summarize(dev_ions(e), (uint32_t)n, (uint32_t)njobs, e->counters.as<unsigned long long>(), e->st), "summary kernel");
    const unsigned long long* cnt = reinterpret_cast<const unsigned long long*>(e->stage.at(StageLayout(njobs).cnt));
    CK(cudaMemcpyAsync(e->stage.at(StageLayout(njobs).cnt), e->counters.p, sizeof(unsigned long long) * mqd::kCounters * njobs,
                       cudaMemcpyDeviceToHost, e->st), "counter download");
    d2h += sizeof(unsigned long long) * mqd::kCounters * njobs;
    if (ions_out && (s = copy_ions(e, ions_out, n, false, &d2h)) != MQ_OK) return s;
    CK(cudaEventRecord(e->ev[1], e->st), "event");
    CK(cudaStreamSynchronize(e->st), "run_batch");
    for (size_t k = 0; k < njobs; ++k) {
        const unsigned long long* c = &cnt[k * mqd::kCounters];
        mq_outcome& o = out[k];
        o.crashed = c[0]; o.returned = c[1]; o.transmitted = c[2]; o.left = c[3]; o.timeout = c[4]; o.n = c[5];
        o.mean_coll = o.n ? (double)c[6] / (double)o.n : 0.0;
        o.mean_time = o.n ? (double)c[7] * ph->dt / (double)o.n : 0.0;
    }
    if (stats) {
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e->ev[0], e->ev[1]);
        stats->kernel_ms = ms;
        stats->ion_steps = steps;
        stats->h2d_bytes = h2d;
        stats->d2h_bytes = d2h;
        stats->kernel_launches += (uint32_t)ntab + 2;   // phase tables + inject + summary
    }
    return MQ_OK;
}

mq_status mq_engine_get_tuning(mq_engine* e, mq_tuning* t) {
    if (!e || !t) return MQ_ERR_INVALID;
    t->threads_per_block = e->tune.tpb;
    t->blocks_per_sm = e->tune.blocks_per_sm;
    t->chunk = e->tune.chunk;
    t->use_graph = e->tune.use_graph;
    t->prefetch = e->tune.prefetch;
    t->wide_records = e->tune.wide;
    t->sort_cells = e->tune.sort_cells;
    return MQ_OK;
}

mq_status mq_engine_set_tuning(mq_engine* e, const mq_tuning* t) {
    if (!e || !t) return MQ_ERR_INVALID;
    if (t->threads_per_block != 128 || t->blocks_per_sm < 1 || t->blocks_per_sm > 3 || t->chunk == 0)
        return fail(e, MQ_ERR_INVALID, "tuning: 128 threads per block, 1..3 blocks per SM, chunk > 0");
    if (t->wide_records && 4 * e->nnodes >= ((size_t)1 << 32))
        return fail(e, MQ_ERR_INVALID, "tuning: wide node records need 4 x nodes below 2^32");
    e->tune.tpb = t->threads_per_block;
    e->tune.blocks_per_sm = t->blocks_per_sm;
    e->tune.chunk = t->chunk;
    e->tune.use_graph = t->use_graph ? 1 : 0;
    e->tune.prefetch = t->prefetch ? 1 : 0;
    e->tune.wide = t->wide_records ? 1 : 0;
    e->tune.sort_cells = t->sort_cells ? 1 : 0;
    return MQ_OK;
}

mq_status mq_engine_inject_fault(mq_engine* e, int32_t kind) {
    if (!e) return MQ_ERR_INVALID;
    if (kind < MQ_FAULT_NONE || kind > MQ_FAULT_LAUNCH) return fail(e, MQ_ERR_INVALID, "unknown fault kind");
    e->fault = kind;
    return MQ_OK;
}

}  // extern "C" (reopened below)

struct MqCheckWordC { unsigned int hits, site; unsigned long long index, limit; };
extern "C" int mq_check_read_f64(MqCheckWordC*, int);
extern "C" int mq_check_read_mixed(MqCheckWordC*, int);
extern "C" int mq_check_read_tandem(MqCheckWordC*, int);
extern "C" int mq_check_read_tandem_mixed(MqCheckWordC*, int);
extern "C" int mq_check_read_probe(MqCheckWordC*, int);
extern "C" int mq_check_selftest_launch(void);

extern "C" {

mq_status mq_check_status(int32_t device, int32_t reset, int32_t* enabled, uint32_t* hits, uint32_t* site,
                          uint64_t* index, uint64_t* limit) {
    if (!enabled || !hits || !site || !index || !limit) return MQ_ERR_INVALID;
    if (mq_device_count() <= device || device < 0) return MQ_ERR_NO_DEVICE;
    int prev = 0;
    cudaGetDevice(&prev);
    if (cudaSetDevice(device) != cudaSuccess) { cudaGetLastError(); return MQ_ERR_CUDA; }
    int (*readers[])(MqCheckWordC*, int) = {mq_check_read_f64, mq_check_read_mixed, mq_check_read_tandem,
                                            mq_check_read_tandem_mixed, mq_check_read_probe};
    *enabled = 0; *hits = 0; *site = 0; *index = 0; *limit = 0;
    mq_status st = MQ_OK;
    for (auto rd : readers) {
        MqCheckWordC w;
        const int r = rd(&w, reset);
        if (r < 0) { st = MQ_ERR_CUDA; break; }
        if (r == 0) *enabled = 1;
        if (w.hits && *hits == 0) { *site = w.site; *index = w.index; *limit = w.limit; }
        *hits += w.hits;
    }
    cudaSetDevice(prev);
    return st;
}

mq_status mq_check_selftest(int32_t device) {
    if (mq_device_count() <= device || device < 0) return MQ_ERR_NO_DEVICE;
    int prev = 0;
    cudaGetDevice(&prev);
    if (cudaSetDevice(device) != cudaSuccess) { cudaGetLastError(); return MQ_ERR_CUDA; }
    const int r = mq_check_selftest_launch();
    cudaSetDevice(prev);
    return r == 0 ? MQ_OK : (r == -3 ? MQ_ERR_NOMEM : MQ_ERR_CUDA);
}

mq_status mq_engine_autotune(mq_engine* e, const mq_job* jobs, size_t njobs, const double dc[4], const mq_physics* ph,
                             uint64_t sample_per_job, mq_tuning* best, double* best_rate) {
    mq_status s = check_batch(e, jobs, njobs, ph);
    if (s != MQ_OK) return s;
    if (e->prec != MQ_PREC_MIXED) return fail(e, MQ_ERR_INVALID, "the autotuner shapes the mixed engine");
    if (sample_per_job == 0) return fail(e, MQ_ERR_INVALID, "sample_per_job must be > 0");
    std::vector<mq_job> sj(jobs, jobs + njobs);
    for (auto& j : sj) j.n = j.n < sample_per_job ? j.n : sample_per_job;
    std::vector<mq_outcome> out(njobs);
    const mqmix::Tuning keep = e->tune;
    mqmix::Tuning top = keep;
    double top_rate = -1.0;
    const int blocks[] = {1, 2, 3};
    const uint32_t chunks[] = {2048, 8192, 20000};
    const int widths = 4 * e->nnodes < ((size_t)1 << 32) ? 2 : 1;
    for (int wd = 0; wd < widths; ++wd)
    for (int pf = 0; pf < 2; ++pf)
    for (int bl : blocks)
        for (uint32_t ch : chunks) {
            e->tune = keep;
            e->tune.blocks_per_sm = bl;
            e->tune.chunk = ch;
            e->tune.prefetch = pf;
            e->tune.wide = wd;
            mq_run_stats st;
            // first call warms the graph and caches; the second is timed
            if ((s = mq_run_batch(e, sj.data(), njobs, dc, ph, out.data(), nullptr, &st)) != MQ_OK) { e->tune = keep; return s; }
            if ((s = mq_run_batch(e, sj.data(), njobs, dc, ph, out.data(), nullptr, &st)) != MQ_OK) { e->tune = keep; return s; }
            double rate = st.step_kernel_ms > 0 ? (double)st.ion_steps / (st.step_kernel_ms * 1e-3) : 0.0;
            if (rate > top_rate) { top_rate = rate; top = e->tune; }
        }
    e->tune = top;
    if (best) mq_engine_get_tuning(e, best);
    if (best_rate) *best_rate = top_rate;
    return MQ_OK;
}

uint64_t mq_fnv1a64(const void* data, size_t bytes, uint64_t h) {
    const unsigned char* p = static_cast<const unsigned char*>(data);
    for (size_t i = 0; i < bytes; ++i) {
        h ^= (uint64_t)p[i];
        h *= 1099511628211ull;
    }
    return h;
}

mq_status mq_summarize(const mq_ions* io, size_t n, double dt, size_t njobs, mq_outcome* out) {
    if (!io || !out || !io->status || !io->jid || !io->ncoll || !io->steps) return MQ_ERR_INVALID;
    std::memset(out, 0, sizeof(mq_outcome) * njobs);
    std::vector<unsigned long long> sc(njobs, 0), ss(njobs, 0);
    for (size_t i = 0; i < n; ++i) {   // summarize, channel.rs:496-506
        uint32_t j = io->jid[i];
        if (j >= njobs) return MQ_ERR_INVALID;
        mq_outcome& o = out[j];
        o.n += 1;
        switch (io->status[i]) {
            case 1: o.crashed += 1; break;
            case 2: o.returned += 1; break;
            case 3: o.transmitted += 1; break;
            case 4: o.left += 1; break;
            default: o.timeout += 1; break;
        }
        sc[j] += io->ncoll[i];
        ss[j] += io->steps[i];
    }
    for (size_t j = 0; j < njobs; ++j)
        if (out[j].n) {
            out[j].mean_coll = (double)sc[j] / (double)out[j].n;
            out[j].mean_time = (double)ss[j] * dt / (double)out[j].n;
        }
    return MQ_OK;
}

}  // extern "C"
