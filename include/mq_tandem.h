/*
 * mq_tandem.h -- C ABI of the nine-channel tandem transport (splitter cube, nine ports,
 * combiner) on the GB300.
 *
 * Reference interfaces replaced (paths inside filiprumenovski/multiq-workbench):
 *   mq_cube_geom, mq_cube_as_built, mq_cube_snap  <- trapsim Geometry::as_built / snap     simulation/trapsim/src/geometry.rs:47-73
 *   mq_cube_classify                             <- Geometry::classify                    simulation/trapsim/src/geometry.rs:136-205
 *   mq_cube_size, mq_cube_port_axis, mq_cube_nearest_port
 *                                                <- size / port_axis_xy / nearest_port    simulation/trapsim/src/geometry.rs:74-125
 *   mq_cube_fields, mq_cube_fields_ex            <- trapsim Fields::build                 simulation/trapsim/src/fields.rs:28-75
 *   mq_cube_dc_combined                          <- Fields::dc_combined                   simulation/trapsim/src/fields.rs:76-86
 *   mq_efield_fieldsolve                         <- fieldsolve Solution::efield_f32       simulation/fieldsolve/src/field.rs:26-87
 *   mq_tandem_create / mq_tandem_destroy         <- trapsim::Model::new (fields, ports)   simulation/trapsim/src/lib.rs:106-175
 *   mq_tandem_inject                             <- the track launch of Model::new        simulation/trapsim/src/lib.rs:131-160
 *   mq_tandem_advance                            <- Model::advance (+ enter / leave)      simulation/trapsim/src/lib.rs:176-276,338-385
 *   mq_tandem_frame                              <- Model::frame (region census)          simulation/trapsim/src/lib.rs:277-336
 */
#ifndef MQ_TANDEM_H
#define MQ_TANDEM_H

#include "mq_engine.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Cube geometry in mm (trapsim Geometry). Port = (axis, side, cell[2]). */
typedef struct mq_cube_geom {
    int32_t n, array;
    double d, pitch, height, t_pcb, gap, stem_r, clear_r, l_ext, ap_r, rod_clear_extra, cap_gap, cap_r;
    int32_t ent_axis, ent_side, ent_cell[2];
    int32_t ext_axis, ext_side, ext_cell[2];
} mq_cube_geom;

#define MQ_CUBE_FREE  0
#define MQ_CUBE_POST  1
#define MQ_CUBE_PLANE 2
#define MQ_CUBE_ENT   3
#define MQ_CUBE_EXT   4

void      mq_cube_as_built(mq_cube_geom* g);
/* spacing pitch/(2 round(pitch/(2 h_target))); plane thickness and port extension snapped to it */
mq_status mq_cube_snap(const mq_cube_geom* g, double h_target, mq_cube_geom* out, double* h);
int32_t   mq_cube_classify(const mq_cube_geom* g, const double p_mm[3], double grow_mm, int32_t* sign);
double    mq_cube_size(const mq_cube_geom* g);
double    mq_cube_post_top_depth(const mq_cube_geom* g);
int32_t   mq_cube_nearest_port(const mq_cube_geom* g, double x_mm, double y_mm);
/* port axis centre (mm) of exit port `index` (index < 0: the entrance) */
mq_status mq_cube_port_axis(const mq_cube_geom* g, int32_t index, double xy_mm[2]);

/* E = -grad(phi) with fieldsolve's stencils (central; one-sided next to electrodes and at the
 * box; electrode nodes from their free neighbours): float4 {Ex, Ey, Ez, phi}. */
mq_status mq_efield_fieldsolve(const double* phi, const uint8_t* mask, int32_t nx, int32_t ny, int32_t nz, double h_m,
                               float* e4);

/* Solve the cube's four bases on the grid of spacing h (mm) with electrode growth grow*h:
 * rf4 = RF E per volt with w = electrode id; wall4 / ent4 / ext4 = DC bases (E, phi).
 * Call with all output pointers NULL to get dims[3] and lo_mm[3] first. */
mq_status mq_cube_fields(const mq_cube_geom* g, double h_mm, double grow, double tol, int32_t threads, int32_t dims[3],
                         double lo_mm[3], float* rf4, float* wall4, float* ent4, float* ext4, mq_solve_stats stats[4]);
/* the same with the Laplace solves on CUDA device `device` (< 0: on the host; same results) */
mq_status mq_cube_fields_ex(const mq_cube_geom* g, double h_mm, double grow, double tol, int32_t threads, int32_t device,
                            int32_t dims[3], double lo_mm[3], float* rf4, float* wall4, float* ent4, float* ext4,
                            mq_solve_stats stats[4]);
/* combined DC for post potential u0 (irrelevant to the force), wall, entrance and exit rods */
mq_status mq_cube_dc_combined(size_t n, const float* wall4, const float* ent4, const float* ext4, double u0,
                              double uwall, double q_in, double q_out, float* out4);

/* ---------------------------------------------------------------- the tandem model */
typedef struct mq_tandem mq_tandem;

/* Per-port counters (trapsim Counts). */
typedef struct mq_port_counts {
    uint32_t entered, returned, forwarded, revisits, from_other;
    uint32_t retry_from[9];
    uint32_t reverse_entries, lost;
    uint32_t by_charge[5];
} mq_port_counts;

/* Species of the track mixture: mass [Da], charge, N2 CCS [A^2], relative abundance. */
typedef struct mq_tandem_species { double mass, z, ccs, weight; } mq_tandem_species;

/* One port's channel: its grid (ports may share one; identical pointers are uploaded once)
 * and its excitation.  tone_khz = 0 marks an idle port: no excitation and gate_bias_v on the
 * gate plate (lib.rs:196-199). */
typedef struct mq_tandem_port {
    int32_t dims[3], pad;
    double h;                          /* [m]                                                */
    const float* rf4;                  /* RF E per volt, w = conductor mask                  */
    const float* ac4;                  /* AC E per volt                                      */
    const float* dc4;                  /* combined DC of the calibrated set                   */
    const float* gate4;                /* gate-plate DC basis per volt                        */
    double tone_khz, v_ac;
} mq_tandem_port;

typedef struct mq_tandem_desc {
    mq_cube_geom cube;                 /* snapped geometry                                   */
    int32_t cube_dims[3], pad0;
    double cube_lo_mm[3], cube_h_mm;
    const float* cube_rf4;             /* RF E per volt (w ignored)                          */
    const float* cube_dc4[2];          /* combined DC: [0] splitter region, [1] combiner      */
    mq_tandem_port port[9];
    double ch_axis_mm, ch_q1_start_mm; /* channel axis (x = y) and Q1 start, shared geometry */
    double v_rf, f_rf, pressure_pa, temp_k, dt;
    double gate_bias_v;                /* 4 V in the reference                                */
    int32_t nspecies;
    int32_t precision;                 /* MQ_PREC_F64: bit-exact FP64 twin of Model::advance;
                                          MQ_PREC_MIXED: FP32 fields, compensated FP32 state,
                                          Philox thermal collisions (statistically equivalent) */
    mq_tandem_species species[8];      /* nspecies <= 5: five charge-state counters per port */
} mq_tandem_desc;

/* Track states (structure of arrays; region 0 splitter, 1..9 port i-1, 10 combiner,
 * 11 lost, 12 back to the source, 13 detected; last = port of the last rejection or -1). */
typedef struct mq_tracks {
    double *x, *y, *z, *vx, *vy, *vz;
    uint64_t* rng;
    int32_t *sp, *region, *last;
} mq_tracks;

typedef struct mq_tandem_frame_counts {
    uint64_t split, channel, combine, lost, back, detected;
} mq_tandem_frame_counts;

mq_status mq_tandem_create(const mq_tandem_desc* d, int32_t device, mq_tandem** out);
void      mq_tandem_destroy(mq_tandem* t);
const char* mq_tandem_last_error(mq_tandem* t);
/* seam height and the nine mouth centres [m] (derived from the description) */
mq_status mq_tandem_layout(const mq_tandem_desc* d, double* seam_m, double* size_m, double mouths_m[18]);
/* launch n tracks as Model::new does (mouth_start: at the nine mouths, else through the entrance) */
mq_status mq_tandem_inject(const mq_tandem_desc* d, uint64_t seed, int32_t mouth_start, mq_tracks* out, size_t n);
/* What one advance executed: track-steps by region kind (splitter/combiner cube, driven port,
 * idle port), kernel time and launches, and the bytes copied each way. */
typedef struct mq_tandem_stats {
    uint64_t steps_cube, steps_port, steps_idle;
    double kernel_ms;
    uint32_t launches, pad;
    uint64_t h2d_bytes, d2h_bytes;
    uint64_t cell_fills_cube;   /* mixed engine: cell-cache fills in the cube (8 x 32-byte records)   */
    uint64_t cell_fills_port;   /* mixed engine: cell-cache fills in the ports (8 x 48-byte records)  */
} mq_tandem_stats;

/* advance tracks (host arrays, in place) by `steps` global steps starting at global step
 * step0; counts[9] accumulate; stats may be NULL.  Synchronous.  With MQ_PREC_MIXED the
 * track's rng word is the key of its counter-based generator and is left unchanged. */
mq_status mq_tandem_advance(mq_tandem* t, mq_tracks* tr, size_t n, uint64_t step0, uint64_t steps,
                            mq_port_counts counts[9], mq_tandem_stats* stats);
mq_status mq_tandem_frame(const mq_tracks* tr, size_t n, mq_tandem_frame_counts* out);

#ifdef __cplusplus
}
#endif
#endif
