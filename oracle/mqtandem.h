/*
 * mqtandem -- CPU oracle for the nine-channel tandem transport.  TEST INFRASTRUCTURE ONLY:
 * used by tests/ and bench.py's CPU baseline for the reference results; the product never
 * links it.
 *
 * A plain-C FP64 restatement of trapsim (filiprumenovski/multiq-workbench):
 *   simulation/trapsim/src/geometry.rs:12-16     electrode ids
 *   simulation/trapsim/src/geometry.rs:47-57     Geometry::as_built
 *   simulation/trapsim/src/geometry.rs:66-125    snap, c0/size/lat, post_valid, n_posts, port_posts,
 *                                                port_axis_xy, port, nearest_port
 *   simulation/trapsim/src/geometry.rs:136-205   Geometry::classify
 *   simulation/trapsim/src/fields.rs:89-96       Fields::grid_coord
 *   simulation/trapsim/src/lib.rs:69-103         cube_field, transport_step
 *   simulation/trapsim/src/lib.rs:106-160        Model::new (seam, mouths, track launch)
 *   simulation/trapsim/src/lib.rs:176-276        Model::advance (drives, region fields, routing)
 *   simulation/trapsim/src/lib.rs:338-385        enter / leave
 *   simulation/mqviz/src/world.rs:265-314        World::fields_at, gate_delta, is_crash
 *   simulation/mqviz/src/world.rs:342-347        SpPhys::new
 *   simulation/mqviz/src/world.rs:407-422        Ion::inject
 *   simulation/mqviz/src/world.rs:473-488        collide
 * Drive values use this library's deterministic sin(2 pi frac(f t)) (mqr_sincos2pi), as the
 * channel oracle does; the reference evaluates libm sin(2 pi f t), which differs in the last
 * bits of the drive value only.
 */
#ifndef MQTANDEM_H
#define MQTANDEM_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mqt_cube {
    int32_t n, array;
    double d, pitch, height, t_pcb, gap, stem_r, clear_r, l_ext, ap_r, rod_clear_extra, cap_gap, cap_r;
    int32_t ent_axis, ent_side, ent_cell[2];
    int32_t ext_axis, ext_side, ext_cell[2];
} mqt_cube;

typedef struct mqt_port {
    int32_t dims[3], pad;
    double h;
    const float *rf4, *ac4, *dc4, *gate4;
    double tone_khz, v_ac;
} mqt_port;

typedef struct mqt_species { double mass, z, ccs, weight; } mqt_species;

typedef struct mqt_desc {
    mqt_cube cube;
    int32_t cube_dims[3], pad0;
    double cube_lo_mm[3], cube_h_mm;
    const float* cube_rf4;
    const float* cube_dc4[2];
    mqt_port port[9];
    double ch_axis_mm, ch_q1_start_mm;
    double v_rf, f_rf, pressure_pa, temp_k, dt;
    double gate_bias_v;
    int32_t nspecies, pad2;
    mqt_species species[8];
} mqt_desc;

typedef struct mqt_tracks {
    double *x, *y, *z, *vx, *vy, *vz;
    uint64_t* rng;
    int32_t *sp, *region, *last;
} mqt_tracks;

#define MQT_NC 21   /* counters per port: entered, returned, forwarded, revisits, from_other,
                       retry_from[9], reverse_entries, lost, by_charge[5] */

void   mqt_as_built(mqt_cube* g);
double mqt_size(const mqt_cube* g);
int    mqt_n_posts(const mqt_cube* g);
int    mqt_classify(const mqt_cube* g, const double p[3], double grow, int32_t* sign);
int    mqt_nearest_port(const mqt_cube* g, double x, double y);
void   mqt_port_axis(const mqt_cube* g, int index, double xy[2]);   /* index < 0: entrance */
void   mqt_layout(const mqt_desc* d, double* seam, double* size, double mouths[18]);
int    mqt_inject(const mqt_desc* d, uint64_t seed, int mouth_start, mqt_tracks* tr, size_t n);
/* routing of one track k (lib.rs:338-385); from_region 0 splitter, 10 combiner */
void   mqt_enter(mqt_tracks* tr, size_t k, int port, int from_region, double seam, const double c[2], double axis,
                 uint32_t counts[MQT_NC]);
void   mqt_leave(mqt_tracks* tr, size_t k, int port, double seam, const double c[2], double axis, uint32_t counts[MQT_NC]);
/* global steps [step0, step0 + steps); counts[9 * MQT_NC] and nsteps[3] (executed track-steps:
 * cube, driven port, idle port; may be NULL) accumulate */
int    mqt_advance(const mqt_desc* d, mqt_tracks* tr, size_t n, uint64_t step0, uint64_t steps,
                   uint32_t* counts, int32_t threads, uint64_t* nsteps);

#ifdef __cplusplus
}
#endif
#endif
