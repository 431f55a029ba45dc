/*
 * mq_engine.h -- C ABI of the GB300 batched ion-trajectory engine.
 *
 * Drop-in for the chsim batch engine of filiprumenovski/multiq-workbench: ion states x
 * operating settings in, per-ion outcome and per-job counts out.  Plain C structs and
 * pointers only; one engine per host thread; every call is synchronous at the ABI and
 * returns an mq_status (never aborts).  Status codes are defined in mq_grid.h.
 *
 * Reference interfaces replaced (paths inside the reference project):
 *   mq_engine_create   <- chsim::channel::Engine::new(fields)        simulation/chsim/src/channel.rs:326-340
 *   mq_engine_destroy  <- Drop of Engine (device buffers, caches)     simulation/chsim/src/channel.rs:309-318
 *   mq_last_error      <- the panics of Engine (expect/assert text)   simulation/chsim/src/channel.rs:328,331,444,446
 *   mq_engine_set_dc   <- Engine::dc_buffer (combined DC field)        simulation/chsim/src/channel.rs:383-395
 *   mq_inject,         <- Engine::inject / mqviz Ion::inject           simulation/chsim/src/channel.rs:342-374,
 *   mq_inject_grid
 *                                                                      simulation/mqviz/src/world.rs:407-422
 *   mq_run_ions        <- Engine::run_batch_ions (states in, states out) simulation/chsim/src/channel.rs:458-475
 *   mq_run_batch       <- Engine::run_batch (jobs in, Outcome per job)  simulation/chsim/src/channel.rs:437-440
 *   mq_summarize       <- summarize                                    simulation/chsim/src/channel.rs:496-506
 *   mq_device_count    <- Device::system_default check                 simulation/chsim/src/channel.rs:328
 *
 * Status per ion (chsim): 0 alive, 1 crashed, 2 returned, 3 transmitted, 4 left box, 5 timeout.
 */
#ifndef MQ_ENGINE_H
#define MQ_ENGINE_H

#include "mq_grid.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mq_engine mq_engine;

#define MQ_PREC_F64   0   /* plain FP64 kernel: bit-exact twin of the FP64 CPU integrator  */
#define MQ_PREC_MIXED 1   /* batched mixed-precision persistent engine                      */

/* Field grid handed to the engine (caller-owned; copied to the device at create).
 * Every array holds nx*ny*nz float4 nodes, index i + nx*(j + ny*k) (chsim Fields). */
typedef struct mq_grid_desc {
    int32_t nx, ny, nz, pad;
    double h;                 /* spacing [m]                                         */
    const float* rf4;         /* RF E per volt, w = conductor mask                   */
    const float* ac4;         /* AC E per volt                                       */
    const float* dc4[4];      /* DC bases per volt: Q1, plate, downstream, box (NULL = zero) */
    double axis_mm;           /* channel axis (x = y)                                */
    double layers_mm[8];      /* layer boundaries l1..l8 (criteria, crash window)    */
} mq_grid_desc;

typedef struct mq_species { double mass, z, ccs_n2; } mq_species;        /* Species, channel.rs:235-240 */
typedef struct mq_rfac { double v_rf, f_rf, v_ac, f_ac; } mq_rfac;       /* RfAc, channel.rs:245-247    */
typedef struct mq_job { mq_species sp; mq_rfac drive; uint64_t n, seed; } mq_job;   /* Job, channel.rs:250-252 */

/* Physics, channel.rs:254-273, plus the launch distribution. */
#define MQ_LAUNCH_DISC     0  /* uniform disc r <= r_inject, Maxwell transverse, flux-weighted v_z */
#define MQ_LAUNCH_LEGACY   1  /* point on axis, 0.1 eV*z*U(0.75,1.5), +-10 deg cone               */
#define MQ_LAUNCH_GAUSSIAN 2  /* Gaussian spot sigma about the axis, Maxwell velocities          */
typedef struct mq_physics {
    int32_t legacy_force, legacy_collisions, legacy_fields, legacy_injection, legacy_criteria;
    int32_t launch;           /* MQ_LAUNCH_*                                          */
    int32_t rf_phase0;        /* 1 = RF phase 0 for every ion (chsim convention)       */
    int32_t pad0;
    double pressure_pa, temp_k, dt, t_max;
    double r_inject_mm, sigma_mm, z_inject_mm;
} mq_physics;

/* Outcome, channel.rs:296-300 */
typedef struct mq_outcome {
    uint64_t n, crashed, returned, transmitted, left, timeout;
    double mean_coll, mean_time;
} mq_outcome;

/* Caller-owned host ion states, structure of arrays (n entries each). */
typedef struct mq_ions {
    double *x, *y, *z, *vx, *vy, *vz;   /* m, m/s                                  */
    double *ph_rf, *ph_ac;              /* drive phase offsets [cycles]             */
    uint64_t* rng;                      /* per-ion random state / key               */
    uint32_t* steps;                    /* executed integrator steps                */
    uint32_t* ncoll;                    /* accepted collisions                      */
    int32_t* leg;                       /* legacy: steps to the next collision      */
    int32_t* status;                    /* chsim status code                        */
    uint32_t* jid;                      /* job index of each ion                    */
} mq_ions;

/* Optional per-call measurements. */
typedef struct mq_run_stats {
    uint64_t ion_steps;        /* executed ion-steps (sum of step counters)          */
    double kernel_ms;          /* device time of the whole call (CUDA events)        */
    uint32_t launches;         /* host-side launch loop iterations / graph replays   */
    uint32_t kernel_launches;  /* kernels of this library launched by the call       */
    uint64_t h2d_bytes, d2h_bytes;
    double step_kernel_ms;     /* device time of the stepping kernel(s) alone        */
    uint32_t step_kernel_launches;
    uint32_t graph_replays;    /* mixed engine: CUDA graph replays of its launch sequence     */
    uint64_t cell_loads;       /* mixed engine: cell-cache fills of the stepping kernel, each
                                  the 8 corner node records of one cell                     */
    uint64_t ions_queued;      /* mixed engine: ions taken from the work queue, summed over the
                                  launches (each reads and writes its working state once)   */
} mq_run_stats;

int32_t     mq_device_count(void);
/* Read bandwidth of the L2 cache on `device` [GB/s]: `passes` read sweeps (L1 bypassed) over a
 * buffer of `bytes` (16 MiB..96 MiB, so it stays resident in L2), timed with CUDA events after one
 * untimed sweep.  The denominator of the gather kernels' L2 roofline; no reference counterpart. */
mq_status   mq_measure_l2_read_gbs(int32_t device, size_t bytes, int32_t passes, double* gbs);
mq_status   mq_engine_create(const mq_grid_desc* grid, int32_t precision, int32_t device, mq_engine** out);
void        mq_engine_destroy(mq_engine* e);
const char* mq_last_error(mq_engine* e);
mq_status   mq_engine_set_dc(mq_engine* e, const double dc[4]);
/* Injection of every job's ions in job order (n = sum of job.n), on the host. */
mq_status   mq_inject(mq_engine* e, const mq_job* jobs, size_t njobs, const mq_physics* ph, mq_ions* out, size_t n);
/* The same injection for a grid without an engine (no device needed). */
mq_status   mq_inject_grid(const mq_grid_desc* grid, const mq_job* jobs, size_t njobs, const mq_physics* ph,
                           mq_ions* out, size_t n);
/* Advance caller states (status 0 ions) by at most max_more steps each (0xFFFFFFFF = to
 * completion) with the DC field last set; states are read and written in place. */
mq_status   mq_run_ions(mq_engine* e, const mq_job* jobs, size_t njobs, const mq_physics* ph, mq_ions* io, size_t n,
                        uint32_t max_more, mq_run_stats* stats);
/* chsim run_batch: inject (on the device), run every ion to completion, count per job.
 * out[njobs] receives the outcomes; ions_out (may be NULL) receives final states.  The FP64
 * engine injects exactly as mq_inject; the mixed engine makes the same random draws (generator
 * state, phases and counters identical) and transforms them to positions and velocities in FP32,
 * the precision the reference's GPU path consumes them in. */
mq_status   mq_run_batch(mq_engine* e, const mq_job* jobs, size_t njobs, const double dc[4], const mq_physics* ph,
                         mq_outcome* out, mq_ions* ions_out, mq_run_stats* stats);
mq_status   mq_summarize(const mq_ions* io, size_t n, double dt, size_t njobs, mq_outcome* out);
/* FNV-1a 64 of `bytes` bytes, continuing from hash `h` (start with 1469598103934665603): the hash
 * chsim's self-check prints over final ion states (fnv, simulation/chsim/src/check.rs:95-99). */
uint64_t    mq_fnv1a64(const void* data, size_t bytes, uint64_t h);

/* Launch shape of the mixed engine (no counterpart in the reference, whose worker shape is
 * fixed by #defines and environment variables: simulation/chsim/src/tiled.rs:10-29). */
typedef struct mq_tuning {
    int32_t threads_per_block;   /* fixed at 128                                          */
    int32_t blocks_per_sm;       /* resident blocks per SM of the persistent grid (1..3)   */
    uint32_t chunk;              /* steps per ion per launch (compaction interval)         */
    int32_t use_graph;           /* replay the launch sequence as one CUDA graph           */
    int32_t prefetch;            /* L1-prefetch the cell each ion is heading for           */
    int32_t wide_records;        /* 64-byte node records read with 256-bit loads (else 48 B;
                                    needs 4 x nodes below 2^32)                            */
    int32_t sort_cells;          /* before every launch, put the live ions in the Morton order
                                    of their cells (a counting sort on the device)         */
} mq_tuning;
mq_status   mq_engine_get_tuning(mq_engine* e, mq_tuning* t);
mq_status   mq_engine_set_tuning(mq_engine* e, const mq_tuning* t);
/* Autotuner: times every candidate shape on a sample of the batch (the first
 * sample_per_job ions of each job), keeps the fastest as the engine's tuning and returns
 * it with its rate in ion-steps/s.  Mixed engine only. */
mq_status   mq_engine_autotune(mq_engine* e, const mq_job* jobs, size_t njobs, const double dc[4], const mq_physics* ph,
                               uint64_t sample_per_job, mq_tuning* best, double* best_rate);

/* Host-side fault injection for tests of the error paths (the reference has none).  The next
 * stepping call of the engine (mq_run_ions / mq_run_batch / mq_engine_autotune) fails once:
 *   MQ_FAULT_LAUNCH_BUDGET  the launch sequence is cut to one launch of 16 steps, so live ions
 *                           remain and the watchdog reports MQ_ERR_WATCHDOG from the real
 *                           survivor count (mq_run_ions still writes the states back: the call
 *                           resumes by calling again);
 *   MQ_FAULT_ALLOC          MQ_ERR_NOMEM before any device allocation of the call;
 *   MQ_FAULT_LAUNCH         MQ_ERR_CUDA in place of the first kernel launch.
 * Nothing is faulted on the device; the engine stays usable.  MQ_FAULT_NONE clears. */
#define MQ_FAULT_NONE          0
#define MQ_FAULT_LAUNCH_BUDGET 1
#define MQ_FAULT_ALLOC         2
#define MQ_FAULT_LAUNCH        3
mq_status   mq_engine_inject_fault(mq_engine* e, int32_t kind);

/* Bounds checks of the debug build (the library built with -DMQ_CHECK): every position-derived
 * gather index and work-queue index of the stepping kernels is checked on the device, and an index
 * out of range is replaced by 0 and recorded.  Reads (and with reset != 0 clears) the records of
 * `device`: *enabled = 1 in a check build, 0 otherwise (then hits = 0); hits = out-of-range
 * indices seen; site / index / limit describe the first.  mq_check_selftest passes one index equal
 * to its limit through the check (no memory access), so a check build must then report a hit at
 * site 99. */
mq_status   mq_check_status(int32_t device, int32_t reset, int32_t* enabled, uint32_t* hits, uint32_t* site,
                            uint64_t* index, uint64_t* limit);
mq_status   mq_check_selftest(int32_t device);

/* ---------------------------------------------------------------------------------------
 * Allocation-free FP64 stepping (no counterpart in the reference).
 *
 * For callers that cannot allocate device memory themselves: code that runs inside a host
 * framework or a plugin host that owns every device allocation (its own pool allocator,
 * a captured or pre-planned memory budget), or that must not call cudaMalloc/cudaFree on
 * the path because those calls synchronise the device.  Such a caller owns the field arrays
 * and the ion states in device memory and passes pointers to them; this call advances the
 * states exactly like mq_run_ions with MQ_PREC_F64 (same kernel, same results bit for bit)
 * and allocates nothing: its working memory (the per-job constant table and two counters)
 * is a fixed array in the library's static device memory, MQ_NOALLOC_SCRATCH_BYTES bytes,
 * which every GPU that loads the library holds until the process exits.
 *
 * Limits and rules:
 *  - njobs <= MQ_NOALLOC_MAX_JOBS; larger batches return MQ_ERR_TOO_LARGE (nothing is run).
 *  - Jobs and physics are checked like every other entry point's (MQ_ERR_INVALID,
 *    MQ_ERR_RF_MISMATCH), and every ion's jid must be < njobs: the call checks that on the
 *    device first and returns MQ_ERR_INVALID, with the states untouched, if one is not.
 *  - The first call on a device looks up the scratch array's device address (once per
 *    device and CUDA context, with that device current); make that first call before any
 *    stream capture.
 *  - All calls share the one scratch array (its contents persist between calls; the call
 *    clears the counters it needs).  Calls that overlap on the GPU - from two host threads,
 *    or on two streams - race on it and must be serialised by the caller.
 *  - The drive phases are evaluated directly each step (the FP64 engine's phase tables are
 *    the same values, precomputed), so no table memory is needed.
 *  - Synchronous: the call waits on `stream` (device-to-host reads of its counters after the
 *    check and after every launch) and returns after the last step, with *ion_steps (may be
 *    NULL) = executed steps.
 */
#define MQ_NOALLOC_MAX_JOBS 4096
#define MQ_NOALLOC_SCRATCH_BYTES (MQ_NOALLOC_MAX_JOBS * 96 + 256)
typedef struct mq_dev_grid {
    int32_t nx, ny, nz, pad;
    double h;                 /* spacing [m]                                        */
    const float* rf4;         /* device: RF E per volt, w = conductor mask          */
    const float* ac4;         /* device: AC E per volt                              */
    const float* dc4;         /* device: combined static DC E (mq_dc_combine)        */
    double axis_mm;
    double layers_mm[8];
} mq_dev_grid;
/* dev_ions: every pointer of the mq_ions struct is a DEVICE pointer (n entries each). */
mq_status   mq_run_ions_device_noalloc(const mq_dev_grid* grid, const mq_job* jobs, size_t njobs, const mq_physics* ph,
                                       const mq_ions* dev_ions, size_t n, uint32_t max_more, void* stream,
                                       uint64_t* ion_steps);

#ifdef __cplusplus
}
#endif
#endif
