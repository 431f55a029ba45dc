/*
 * mq_fit.h -- resonance-curve fits and the secular-frequency terrain (C ABI).
 *
 * The callers that turn per-frequency outcome counts of a batch sweep into a
 * resolving power R = f0 / FWHM (and R in m/z terms): a weighted, bounded
 * Levenberg-Marquardt fit of a Lorentzian or Gaussian on a flat baseline to
 * binomial counts, with model-based variances, a covariance error on R and a
 * parametric bootstrap; and the principal-axis gradient tables along the
 * channel axis that give the local Mathieu secular frequency of a species
 * (used for d f / d(m/z)).  All host code; deterministic (no FMA contraction).
 *
 * Reference interfaces replaced (paths inside filiprumenovski/multiq-workbench):
 *   mq_fit_model              <- fit::model, Shape::g                    simulation/mqviz/src/fit.rs:13-33
 *   mq_fit_shape_sigma        <- fit::fit_shape_sigma                    simulation/mqviz/src/fit.rs:185-191
 *   mq_fit_binomial_shape     <- fit::fit_binomial_shape                 simulation/mqviz/src/fit.rs:211-246
 *   mq_fit_binomial_curve     <- fit::fit_binomial_curve                 simulation/mqviz/src/fit.rs:249-255
 *   mq_fit_is_significant     <- fit::is_significant (+ MIN_DELTA_CHI2)  simulation/mqviz/src/fit.rs:257-265
 *   mq_fit_r_mz               <- fit::r_mz                               simulation/mqviz/src/fit.rs:268-272
 *   mq_rng_*                  <- stats::Rng (xorshift64, binomial)       simulation/mqviz/src/stats.rs:152-171
 *   mq_mathieu_beta           <- terrain::beta                           simulation/mqviz/src/terrain.rs:6-23
 *   mq_sec_freq_khz           <- terrain::sec_freq_khz                   simulation/mqviz/src/terrain.rs:25-30
 *   mq_terrain_tables         <- the terrain-table block of World::build_calibrated
 *                                                                        simulation/mqviz/src/world.rs:187-231
 *   mq_terrain_compute        <- terrain::compute                        simulation/mqviz/src/terrain.rs:40-55
 *   mq_terrain_dfdmz          <- analysis::dfdmz                         simulation/mqviz/src/analysis.rs:10-18
 *   mq_secular_freq           <- chsim secular_freq                      simulation/chsim/src/channel.rs:555-578
 */
#ifndef MQ_FIT_H
#define MQ_FIT_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MQ_SHAPE_LORENTZ 0
#define MQ_SHAPE_GAUSS   1
#define MQ_FIT_MIN_DELTA_CHI2 16.0

/* One fitted resonance: y = b + A g((f - f0) / w), p = [b, A, f0, w], w the FWHM. */
typedef struct mq_res_fit {
    int32_t shape;          /* MQ_SHAPE_*                                                     */
    int32_t converged;
    double p[4];            /* b, A, f0, w                                                    */
    double e[4];            /* 1-sigma errors of p                                            */
    double cov[16];         /* row-major covariance, scaled by max(1, chi2/dof)               */
    double chi2;
    double chi2_flat;       /* chi2 of the flat model (NaN when not computed)                 */
    int64_t dof;
    double scale;           /* max(1, sqrt(chi2/dof))                                         */
    uint64_t n_pts;
    double r, r_err;        /* R = f0 / w, delta-method error with the full covariance        */
    int32_t has_boot, pad;
    double r_boot_mean, r_boot_sd, f0_boot_sd;   /* parametric bootstrap (has_boot != 0)      */
} mq_res_fit;

/* Peak-normalised model value at x. */
double mq_fit_model(int32_t shape, const double p[4], double x);

/* Fit one shape with given sigma_i.  0 on success, MQ_ERR_INVALID (-1) when the inputs are
 * malformed or fewer than 6 points, 1 when no fit is possible (singular normal equations). */
int32_t mq_fit_shape_sigma(int32_t shape, const double* xs, const double* ys, const double* sg, size_t n,
                           mq_res_fit* out);

/* Fit one shape to k successes of n at each x (points with n = 0 are dropped; at least 6 must
 * remain), variances from the fitted model iterated three times, `boot` bootstrap replicas
 * seeded with seed ^ 0xB007.  Return codes as mq_fit_shape_sigma. */
int32_t mq_fit_binomial_shape(int32_t shape, const double* xs, const uint64_t* ks, const uint64_t* ns, size_t n,
                              uint64_t boot, uint64_t seed, mq_res_fit* out);

/* Both shapes; the lower chi2 wins (the Lorentzian on a tie). */
int32_t mq_fit_binomial_curve(const double* xs, const uint64_t* ks, const uint64_t* ns, size_t n, uint64_t boot,
                              uint64_t seed, mq_res_fit* out);

/* 1 if the fit beats the flat curve by MQ_FIT_MIN_DELTA_CHI2 and is well posed over xs, else 0. */
int32_t mq_fit_is_significant(const mq_res_fit* f, const double* xs, size_t n);

/* FWHM in frequency -> (delta m/z, its error, R_mz, its error) for slope dfdmz [kHz per m/z]. */
void mq_fit_r_mz(double mz, double dfdmz, double fwhm, double fwhm_err, double out[4]);

/* The statistics generator: state = seed * 0x9E3779B97F4A7C15 | 1, xorshift64 (13, 7, 17). */
uint64_t mq_rng_seed(uint64_t seed);
double mq_rng_uniform(uint64_t* state);
/* out[i] = binomial(n[i], p[i]) drawn in order i = 0..m-1 (normal approximation above n = 400 and
 * n p (1 - p) > 50, as the reference). */
void mq_rng_binomial_fill(uint64_t* state, const uint64_t* n, const double* p, size_t m, uint64_t* out);

/* Mathieu characteristic exponent beta(a, q), first stability region. */
double mq_mathieu_beta(double a, double q);
/* Secular frequency [kHz] for principal RF / DC gradients [V/m^2 per volt], q/m [C/kg], RF amplitude
 * and frequency; NaN outside the first stability region (a + q^2/2 <= 0 or q > 0.95). */
double mq_sec_freq_khz(double g_rf, double g_dc, double qm, double v_rf, double f_rf);

/* Principal-axis gradient tables on the channel axis (x = y = axis_m) at z = 0.3 mm, 0.4 mm, ...
 * while z < min((nz - 2) h, 20 mm): per z the RF Jacobian's principal directions and the RF and
 * four DC-basis second derivatives along them.  rf4 and dc4[b] are float4 node arrays (E per volt,
 * w ignored).  Writes up to `cap` rows: z_mm[k], rf2[2k + {0,1}], dc2[(b * cap + k) * 2 + {0,1}];
 * *n_out = rows written.  MQ_ERR_INVALID when cap is too small. */
int32_t mq_terrain_tables(int32_t nx, int32_t ny, int32_t nz, double h, double axis_m, const float* rf4,
                          const float* const dc4[4], size_t cap, double* z_mm, double* rf2, double* dc2, size_t* n_out);

/* Secular frequencies fx, fy [kHz] of species s (mass [Da], z) along the table:
 * fx[s * n + k], fy[s * n + k]; dc2 laid out as mq_terrain_tables with stride `cap`. */
int32_t mq_terrain_compute(size_t n, size_t cap, const double* rf2, const double* dc2, const double* mass,
                           const double* charge, size_t nsp, double v_rf, const double dc[4], double f_rf,
                           double* fx, double* fy);

/* d f_sec / d(m/z) [kHz per m/z] at the body plateau (first z >= 6 mm, x mode) by the central
 * difference of m -> m (1 +- 1 %). */
double mq_terrain_dfdmz(size_t n, size_t cap, const double* z_mm, const double* rf2, const double* dc2, double mass,
                        double charge, double v_rf, const double dc[4], double f_rf);

/* Secular frequency [Hz] from a trajectory (chsim secular_freq, simulation/chsim/src/channel.rs:555-578):
 * an FP64 ion of charge-to-mass qm [C/kg] released at rest 0.2 mm off the axis (x = y = axis_m) along
 * (1, -1)/sqrt2 in the z = z_m slice of the RF field (rf4: float4 E per volt, grid spacing h [m]),
 * driven by v_rf sin(2 pi f_rf t) with the transverse force only, 200 steps per RF period for 4 ms;
 * the frequency of the upward zero crossings of x - y.  *out = NaN when the ion leaves the 2.5 mm
 * window or crosses fewer than three times.  Indices are clamped to the grid. */
int32_t mq_secular_freq(const float* rf4, int32_t nx, int32_t ny, int32_t nz, double h, double axis_m, double qm,
                        double v_rf, double f_rf, double z_m, double* out);

#ifdef __cplusplus
}
#endif
#endif
