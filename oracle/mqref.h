/*
 * mqref -- CPU oracle for the batched ion-trajectory path.  TEST INFRASTRUCTURE ONLY:
 * used by tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference arm
 * as the reference results of the parity tests and the timed host baseline.  The product
 * never links or calls it.
 *
 * A plain-C FP64 restatement of the reference integrator of filiprumenovski/multiq-workbench:
 *   simulation/mqviz/src/world.rs:265-288   World::fields_at (one pass over 8 corners)
 *   simulation/mqviz/src/world.rs:308-314   World::is_crash (box, nearest-node mask)
 *   simulation/mqviz/src/world.rs:385-422   xs_next / gs / splitmix / Ion::inject
 *   simulation/mqviz/src/world.rs:437-465   Clock::fill (global phase per step)
 *   simulation/mqviz/src/world.rs:471-488   collide (null-collision Maxwell N2 bath)
 *   simulation/mqviz/src/world.rs:498-536   advance_with_field (kick, drift, collide, tests)
 *   simulation/mqviz/src/world.rs:538-549   advance_all (work split in chunks of 16 ions)
 *   simulation/mqviz/src/validate.rs:24-46  run_live seeding splitmix(seed + i*0x9E37)
 *   simulation/mqviz/src/validate.rs:49-94  run_reference, the independent per-ion form
 *   simulation/mqviz/src/world.rs:110-131   tri_one (one field per trilinear pass)
 * with chsim's physics switches restated in FP64:
 *   simulation/chsim/src/channel.rs:254-273  Physics (legacy / correct presets)
 *   simulation/chsim/src/channel.rs:342-381  inject (legacy point+cone launch, first free path)
 *   simulation/chsim/src/channel.rs:397-426  batch_params / job_params (qm_kick x0.5 legacy,
 *                                            criteria, crash window, gas constants)
 *   simulation/chsim/src/channel.metal:56-62,100-119 nearest-node fields, legacy stationary-gas
 *                                            collisions, termination tests
 *   simulation/chsim/src/channel.rs:496-506  summarize
 *
 * Status codes follow chsim: 0 alive, 1 crashed (electrode), 2 returned, 3 transmitted,
 * 4 left box, 5 timeout.
 *
 * Transcendentals are this file's own deterministic implementations (atanh-series log,
 * Taylor sin/cos after exact turn-based range reduction) compiled without FMA
 * contraction, so results are identical on any host and reproducible by an FP64 GPU
 * kernel that evaluates the same operations in the same order.
 */
#ifndef MQREF_H
#define MQREF_H
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mqr_grid {
    int32_t nx, ny, nz;
    double h;                 /* spacing [m] */
    const float* rf4;         /* RF E per volt, w = conductor mask (float4 per node) */
    const float* ac4;         /* AC E per volt                                       */
    const float* dc4;         /* combined static DC E                                 */
} mqr_grid;

typedef struct mqr_batch {
    int32_t legacy_force, legacy_collisions, legacy_fields, legacy_injection, legacy_criteria;
    int32_t launch;           /* 0 effusive disc, 1 legacy point + cone, 2 Gaussian spot */
    int32_t rf_phase0;        /* 1: every ion starts at RF phase 0 (chsim convention)   */
    int32_t pad0;
    double pressure_pa, temp_k, dt, t_max;
    double r_inject_mm;       /* disc radius (launch 0)                                 */
    double sigma_mm;          /* Gaussian spot sigma (launch 2)                          */
    double z_inject_mm;       /* launch plane                                           */
    double v_rf, f_rf;        /* RF drive shared by the batch                            */
    double axis_mm;           /* channel axis x = y                                      */
    double layers_mm[8];      /* geometry layer boundaries l1..l8                        */
} mqr_batch;

typedef struct mqr_job {
    double mass, z, ccs_n2;   /* Da, charge number, N2 CCS [A^2] */
    double v_ac, f_ac;
    uint64_t n, seed;
} mqr_job;

typedef struct mqr_ions {
    double *x, *y, *z, *vx, *vy, *vz;   /* m, m/s                                  */
    double *ph_rf, *ph_ac;              /* phase offsets [cycles, 0..1)            */
    uint64_t* rng;                      /* xorshift64 state                         */
    uint32_t* steps;                    /* executed steps                           */
    uint32_t* ncoll;                    /* accepted collisions                      */
    int32_t* leg;                       /* legacy: steps to the next collision      */
    int32_t* status;
    uint32_t* jid;
} mqr_ions;

typedef struct mqr_outcome {
    uint64_t n, crashed, returned, transmitted, left, timeout;
    double mean_coll, mean_time;
} mqr_outcome;

/* deterministic math (exported for tests) */
double mqr_log(double x);
void   mqr_sincos2pi(double u, double* s, double* c);
uint64_t mqr_splitmix(uint64_t z);

/* number of steps an ion may take: round(t_max / dt) */
uint32_t mqr_max_steps(const mqr_batch* b);

/* inject every job's ions (job order), writing n = sum(job.n) ions */
int mqr_inject(const mqr_batch* b, const mqr_job* jobs, size_t njobs, mqr_ions* ions, size_t n);

/* advance every ion with status 0 until it finishes; returns executed ion-steps in *steps_out */
int mqr_run(const mqr_grid* g, const mqr_batch* b, const mqr_job* jobs, size_t njobs,
            mqr_ions* ions, size_t n, int32_t threads, uint64_t* steps_out);

/* same as mqr_run, but only ions [i0, i1) and each ion at most max_steps more steps */
int mqr_run_range(const mqr_grid* g, const mqr_batch* b, const mqr_job* jobs, size_t njobs,
                  mqr_ions* ions, size_t i0, size_t i1, uint32_t max_more, int32_t threads,
                  uint64_t* steps_out);

int mqr_summarize(const mqr_ions* ions, size_t n, const mqr_batch* b, size_t njobs, mqr_outcome* out);

/* The independent per-ion form of validate.rs:49-94 (a cross-check of the table-driven integrator):
 * own seeding ((id + 1) * golden ^ seed), own time accumulator t += dt, drive sin(2 pi (f t + phase))
 * each step, a separate trilinear pass per field (world.rs:112-131), collisions inline, exit ->
 * return -> crash tests, timeout at t_max.  Phases are drawn in turns (the reference draws radians,
 * 2 pi u) and its sine is this library's turn-based one. */
typedef struct mqr_indep {
    double mass, z, ccs_n2;   /* Da, charge, N2 CCS [A^2]                 */
    double v_rf, f_rf, v_ac, f_ac;
    double pressure_pa, dt, t_max;
    double axis_mm, z_exit, z_return;   /* [mm], [m], [m]               */
    uint64_t seed;
    int32_t rf_phase0, pad;
} mqr_indep;

typedef struct mqr_counts { uint64_t n, transmitted, crashed, returned, timeout, steps; } mqr_counts;

int mqr_run_independent(const mqr_grid* g, const mqr_indep* p, uint64_t n, int32_t threads, mqr_counts* out);

#ifdef __cplusplus
}
#endif
#endif
