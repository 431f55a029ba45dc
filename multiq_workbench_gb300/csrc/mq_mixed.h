// Mixed-precision batched engine (internal interface; see mq_mixed.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "mq_internal.h"

namespace mqmix {

// Per-job constants of the mixed kernel.  Positions are held in grid units (cells) and
// velocities in cells per step, so the kick is E [V/m] * qm_kick * dt^2 / h.
struct MixJob {
    float kick;        // qm_kick * dt * dt / h
    float v_ac;        // AC amplitude [V]
    float cand_a;      // null-collision candidate probability per |u| (nsd * h / dt)
    float cand_b;      //   ... constant part (nsd * E|V|, E|V| = 2 sqrt(2/pi) s_gas: mqx::thermal_partner)
    float s_gas;       // Maxwell gas std [m/s]
    float mr;          // M_gas / (m + M_gas)
    float floor_v;     // legacy: no collision below this speed [m/s]; < 0 = thermal gas
    float mfp_mean;    // legacy mean free path [m]
    uint32_t w_ac_lo, w_ac_hi;   // AC phase increment per step, turns * 2^64
    float cw_ac, sw_ac;          // cos / sin of the AC phase advance per step
    int32_t use_ac;
    int32_t pad;
};

struct MixBatch {      // per-batch constants (device-resident parameter block)
    double h, inv_h, dt, u2v, v2u;   // u2v = h / dt (cells/step -> m/s)
    float v_rf, dt_f, u2v_f, v2u_f;
    uint32_t w_rf_lo, w_rf_hi;       // RF phase increment per step, turns * 2^64
    float cw_rf, sw_rf;              // cos / sin of the RF phase advance per step
    float z_exit_h, z_exit_l, z_ret_h, z_ret_l;       // grid units, double-float
    float cz0_h, cz0_l, cz1_h, cz1_l;                 // crash window, grid units
    float z_exit_near, z_ret_near;                    // one cell inside the exit / return planes
    float lim_x, lim_y, lim_z;                        // n - 1 (exact)
    int32_t nx, ny, nz;
    int32_t nearest, legacy_coll;
    uint32_t max_steps;
    int32_t pad;
};

struct Tuning {
    int tpb = 128;             // threads per block
    int blocks_per_sm = 3;     // resident blocks per SM for the persistent grid (168 registers/thread; 3 at most);
                               // the nearest-node kernels (about 100 registers) run as many as fit instead
    uint32_t chunk = 20000;    // steps per ion per launch (compaction interval)
    int use_graph = 1;         // replay the launch sequence as one CUDA graph
    int prefetch = 0;          // L1-prefetch the cell an ion is heading for
    int wide = 0;              // 64-byte node records read with 256-bit loads (else 48-byte records)
    uint32_t max_launches = 0; // cap on launches per call (0 = as many as the step budget needs)
    int sort_cells = 0;        // put each launch's live list in the Morton order of the ions' cells
    int sms = 0;               // filled from the device
};

struct Scratch {
    void* lists = nullptr;     // two live-ion lists (ping-pong), u32 each
    size_t list_cap = 0;
    void* ctrs = nullptr;      // counters: [0] head, [1..2] counts, [4..5] steps (u64), ...
    void* params = nullptr;    // MixBatch
    void* jobs = nullptr;      // MixJob[]
    size_t jobs_cap = 0;
    void* keep = nullptr;      // working state of the call's ions (phase offsets, double-floats, staged flags)
    size_t keep_cap = 0;
    void* nodes = nullptr;     // interleaved RF | DC | AC node records (float4 x 3 or 4 per node)
    size_t nodes_cap = 0;
    uint64_t nodes_gen = ~0ull; // grid generation the records were packed from
    int nodes_stride = 0;       // float4 per record of the packed records
    void* sort = nullptr;      // cell sort: bin counts, tile totals, keys and the sorted list
    size_t sort_cap = 0;
    cudaGraphExec_t graph = nullptr;
    uint64_t graph_key[6] = {0, 0, 0, 0, 0, 0};
    cudaEvent_t ev[2] = {nullptr, nullptr};
};

struct RunInfo {
    uint64_t ion_steps = 0;
    uint64_t cell_loads = 0;   // cell-cache fills of the stepping kernel (8 node records each)
    uint64_t ions_queued = 0;  // ions taken from the work queue, summed over the launches
    float step_ms = 0.0f;
    uint32_t step_launches = 0;
    uint32_t kernel_launches = 0;
    uint32_t graph_replays = 0;
    int watchdog = 0;
    uint32_t survivors = 0;
};

MixJob make_mix_job(const mqp::JobC& j, const mqp::Batch& b);
MixBatch make_mix_batch(const mqp::Batch& b);
// device injection of a batch for the mixed engine: the FP64 injection's draws with FP32 transforms
cudaError_t launch_inject(const mqp::Batch& b, mqd::JobTable jt, mqd::DevIons io, uint32_t n, cudaStream_t st);
Tuning default_tuning(int device, size_t nodes);
// write_states = 0 leaves the FP64 position / velocity of the ion states as they were (a caller
// that wants only the counters, steps, status and collision counts)
cudaError_t run(Scratch& s, const Tuning& t, mqd::DevGrid g, uint64_t grid_gen, const mqp::Batch& b, const MixJob* jobs,
                size_t njobs, mqd::DevIons io, uint32_t n, uint32_t max_more, int write_states, cudaStream_t st,
                RunInfo* info);
void release(Scratch& s);

}  // namespace mqmix
