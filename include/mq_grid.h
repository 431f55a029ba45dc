/*
 * mq_grid.h -- field-grid set-up for the batched ion-trajectory engine (C ABI).
 *
 * Produces the per-volt basis fields the engine steps ions through: the
 * ejection-channel geometry rasteriser, a Laplace solver for masked Dirichlet
 * grids, E = -grad(phi) and the combined static DC field.  All functions are
 * CPU code; they are deterministic (no FMA contraction, thread-count-independent
 * reductions) so a grid built on any host is bit-identical.
 *
 * Reference interfaces replaced (paths inside filiprumenovski/multiq-workbench):
 *   mq_geom / mq_geom_default     <- chsim::channel::Geom + Default      simulation/chsim/src/channel.rs:18-44
 *   mq_geom_dims, mq_geom_axis_mm <- Geom::nz / Geom::axis               simulation/chsim/src/channel.rs:55-59
 *   mq_geom_classify              <- Geom::classify                      simulation/chsim/src/channel.rs:61-101
 *   mq_geom_basis_problem         <- solve_basis's Problem::from_fn + basis_value
 *                                                                         simulation/chsim/src/channel.rs:111-120,143-151
 *   mq_laplace_solve              <- fieldsolve::solve                   simulation/fieldsolve/src/lib.rs:156-166
 *   mq_laplace_solve_device       <- the same solve on the GPU (no counterpart in the reference, which solves on the CPU)
 *   mq_efield_central             <- chsim efield (central differences)  simulation/chsim/src/channel.rs:167-184
 *   mq_channel_basis              <- solve_basis + efield (+ RF mask)    simulation/chsim/src/channel.rs:143-165,204-217
 *   mq_channel_basis_ex           <- the same with the solve on a chosen device
 *   mq_dc_combine                 <- Fields::dc_field                    simulation/chsim/src/channel.rs:219-226
 */
#ifndef MQ_GRID_H
#define MQ_GRID_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes shared by every entry point of this library (mq_engine.h uses the same values). */
typedef int32_t mq_status;
#define MQ_OK              0
#define MQ_ERR_INVALID    -1   /* bad argument (null pointer, size, value out of range)        */
#define MQ_ERR_CUDA       -2   /* a CUDA runtime call failed                                    */
#define MQ_ERR_NOMEM      -3   /* host or device allocation failed                              */
#define MQ_ERR_WATCHDOG   -4   /* a device loop hit its iteration cap and returned early        */
#define MQ_ERR_RF_MISMATCH -5  /* jobs of one batch do not share one RF drive                   */
#define MQ_ERR_NO_DEVICE  -6   /* no CUDA device visible                                        */
#define MQ_ERR_NOT_CONVERGED -7 /* Laplace solve did not reach its tolerance                    */
#define MQ_ERR_TOO_LARGE  -8   /* request exceeds a fixed capacity of the entry point           */

/* Channel geometry, all lengths in mm (field meaning as in chsim Geom). */
typedef struct mq_geom {
    double de;          /* rod diameter                                   */
    double coef;        /* gap / De                                       */
    double q1_start;
    double q1_len;
    double alpha;       /* squeeze per mm of z                            */
    double gap;
    double plate;
    double hole_d;
    double q2_len;
    double stem_d;
    int32_t q2_flare_bug;  /* Q2 reuses the Q1 squeeze formula            */
    int32_t tilt_mode;     /* 0 code, 1 paper/inset, 2 symmetric squeeze  */
    int32_t ac_mode;       /* 0 code: all Q1 rods, 1 paper: lower pair    */
    int32_t n_xy;          /* nodes per transverse axis                   */
    double grow;        /* convex electrodes grown by grow*h              */
    double h_mm;        /* grid spacing                                   */
    double mis[4][4];   /* per Q1 rod [LL,RL,LU,RU]: dx, dy, dx/dz, dy/dz */
} mq_geom;

/* Basis identifiers (chsim Basis). */
#define MQ_BASIS_RF       0
#define MQ_BASIS_AC       1
#define MQ_BASIS_DC_Q1    2
#define MQ_BASIS_DC_PLATE 3
#define MQ_BASIS_DC_DOWN  4
#define MQ_BASIS_DC_BOX   5

/* Electrode codes written by mq_geom_classify: 0 free; else 1 + kind*4 + quadrant with
 * kind 0 Q1, 1 Stem3, 2 Plate, 3 Stem5, 4 Q2, 5 Stem7, 6 Slab (quadrant 0 for Plate/Slab). */
#define MQ_ELEC_NONE 0

typedef struct mq_solve_stats {
    int32_t iterations;      /* preconditioned CG iterations                              */
    int32_t converged;       /* final_residual <= tol                                     */
    double final_residual;   /* max_free |sum of 6 neighbours - 6 phi| / max(|fixed|,|outer|) */
    double seconds;
} mq_solve_stats;

void      mq_geom_default(mq_geom* g);
/* Grid dimensions nx, ny, nz of the geometry (nz = z_len/h). */
mq_status mq_geom_dims(const mq_geom* g, int32_t dims[3]);
/* Channel axis coordinate (x = y = axis) in mm, and the 8 layer boundaries l1..l8 in mm. */
double    mq_geom_axis_mm(const mq_geom* g);
void      mq_geom_layers(const mq_geom* g, double layers[8]);
/* Electrode code per node, index i + nx*(j + ny*k). */
mq_status mq_geom_classify(const mq_geom* g, uint8_t* elec, size_t n);
/* Dirichlet problem of one basis: mask (1 = electrode) and fixed potential per node,
 * plus the outer-face potential it is solved with (1 V for the box basis, else 0). */
mq_status mq_geom_basis_problem(const mq_geom* g, int32_t basis, uint8_t* mask, double* fixed,
                                size_t n, double* outer_bc);

/* Laplace solve on a masked Dirichlet grid. Box faces are Dirichlet at outer_bc unless
 * masked.  Stops when the scaled true max-norm residual <= tol.  phi receives the
 * potential (length nx*ny*nz).  threads <= 0 uses every hardware thread. */
mq_status mq_laplace_solve(int32_t nx, int32_t ny, int32_t nz, const uint8_t* mask,
                           const double* fixed, double outer_bc, double tol, int32_t threads,
                           double* phi, mq_solve_stats* stats);
/* mq_laplace_solve on CUDA device `device`: the same algorithm and the same floating-point
 * operations in the same order, so the potential is bit-identical to the host solver's. */
mq_status mq_laplace_solve_device(int32_t nx, int32_t ny, int32_t nz, const uint8_t* mask, const double* fixed,
                                  double outer_bc, double tol, int32_t device, double* phi, mq_solve_stats* stats);

/* E = -grad(phi) per node as float4 {Ex, Ey, Ez, 0}: central differences, one-sided at
 * the box faces.  h_m = spacing in metres. */
mq_status mq_efield_central(const double* phi, int32_t nx, int32_t ny, int32_t nz, double h_m,
                            float* e4);

/* Solve one channel basis and write its float4 field (RF: w = conductor mask).
 * phi_out may be NULL. */
mq_status mq_channel_basis(const mq_geom* g, int32_t basis, double tol, int32_t threads,
                           float* e4, double* phi_out, mq_solve_stats* stats);
/* the same with the Laplace solve on CUDA device `device` (< 0: on the host) */
mq_status mq_channel_basis_ex(const mq_geom* g, int32_t basis, double tol, int32_t threads, int32_t device,
                              float* e4, double* phi_out, mq_solve_stats* stats);

/* Combined static DC field out4[n] = sum_b (float)v[b] * dc4[b][n] in float, bases in
 * order 0..3 (a NULL basis contributes nothing). */
mq_status mq_dc_combine(size_t n, const float* const dc4[4], const double v[4], float* out4);

#ifdef __cplusplus
}
#endif
#endif
