/*
 * mqref.c -- CPU oracle (TEST INFRASTRUCTURE ONLY; see mqref.h for the reference
 * functions restated here, file:line in filiprumenovski/multiq-workbench).
 *
 * Build: gcc -O2 -std=c11 -ffp-contract=off -fPIC -pthread -shared mqref.c -o _ref/libmqref.so
 * (-ffp-contract=off keeps every a*b+c as two rounded operations on every host, which is
 * what makes the results reproducible on x86-64 and aarch64 alike.)
 */
#define _GNU_SOURCE
#include "mqref.h"

#include <math.h>
#include <unistd.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* physical constants: simulation/chsim/src/channel.rs:11-14, simulation/mqviz/src/world.rs:13-16 */
static const double AMU = 1.6605390666e-27;
static const double QE = 1.602176634e-19;
static const double KB = 1.380649e-23;

/* ------------------------------------------------------------------ deterministic math */

/* sin/cos Taylor coefficients (-1)^k/(2k+1)!, (-1)^k/(2k)!  (correctly rounded) */
#define S1 (-0x1.5555555555555p-3)
#define S2 (0x1.1111111111111p-7)
#define S3 (-0x1.a01a01a01a01ap-13)
#define S4 (0x1.71de3a556c734p-19)
#define S5 (-0x1.ae64567f544e4p-26)
#define S6 (0x1.6124613a86d09p-33)
#define S7 (-0x1.ae7f3e733b81fp-41)
#define S8 (0x1.952c77030ad4ap-49)
#define C2 (0x1.5555555555555p-5)
#define C3 (-0x1.6c16c16c16c17p-10)
#define C4 (0x1.a01a01a01a01ap-16)
#define C5 (-0x1.27e4fb7789f5cp-22)
#define C6 (0x1.1eed8eff8d898p-29)
#define C7 (-0x1.93974a8c07c9dp-37)
#define C8 (0x1.ae7f3e733b81fp-45)
#define C9 (-0x1.6827863b97d97p-53)
#define PIO2 (0x1.921fb54442d18p+0)
/* atanh series coefficients 1/(2k+1), k = 1..11 */
#define L1 (0x1.5555555555555p-2)
#define L2 (0x1.999999999999ap-3)
#define L3 (0x1.2492492492492p-3)
#define L4 (0x1.c71c71c71c71cp-4)
#define L5 (0x1.745d1745d1746p-4)
#define L6 (0x1.3b13b13b13b14p-4)
#define L7 (0x1.1111111111111p-4)
#define L8 (0x1.e1e1e1e1e1e1ep-5)
#define L9 (0x1.af286bca1af28p-5)
#define L10 (0x1.8618618618618p-5)
#define L11 (0x1.642c8590b2164p-5)
#define LN2_HI (0x1.62e42fee00000p-1)
#define LN2_LO (0x1.a39ef35793c76p-33)
#define SQRT_HALF (0x1.6a09e667f3bcdp-1)

static inline double sin_k(double x) {
    double z = x * x;
    double p = S7 + z * S8;
    p = S6 + z * p;
    p = S5 + z * p;
    p = S4 + z * p;
    p = S3 + z * p;
    p = S2 + z * p;
    p = S1 + z * p;
    return x + (x * z) * p;
}
static inline double cos_k(double x) {
    double z = x * x;
    double p = C8 + z * C9;
    p = C7 + z * p;
    p = C6 + z * p;
    p = C5 + z * p;
    p = C4 + z * p;
    p = C3 + z * p;
    p = C2 + z * p;
    return (1.0 - 0.5 * z) + (z * z) * p;
}

/* sin and cos of 2*pi*u: exact reduction in turns (4u - nearest integer), then Taylor. */
void mqr_sincos2pi(double u, double* s, double* c) {
    u = u - floor(u);
    double t = 4.0 * u;
    double q = nearbyint(t);
    double x = (t - q) * PIO2;
    double sk = sin_k(x), ck = cos_k(x);
    int qi = ((int)q) & 3;
    switch (qi) {
        case 0: *s = sk; *c = ck; break;
        case 1: *s = ck; *c = -sk; break;
        case 2: *s = -sk; *c = -ck; break;
        default: *s = -ck; *c = sk; break;
    }
}

/* natural log for finite x > 0: x = m 2^e, m in [sqrt(1/2), sqrt(2)), log m = 2 atanh(s), s = (m-1)/(m+1) */
double mqr_log(double x) {
    int e;
    double m = frexp(x, &e);
    if (m < SQRT_HALF) { m = m * 2.0; e -= 1; }
    double f = m - 1.0;
    double s = f / (2.0 + f);
    double z = s * s;
    double r = L10 + z * L11;
    r = L9 + z * r;
    r = L8 + z * r;
    r = L7 + z * r;
    r = L6 + z * r;
    r = L5 + z * r;
    r = L4 + z * r;
    r = L3 + z * r;
    r = L2 + z * r;
    r = L1 + z * r;
    double ls = 2.0 * s;
    double lm = ls + (ls * z) * r;
    double de = (double)e;
    return (de * LN2_LO + lm) + de * LN2_HI;
}

uint64_t mqr_splitmix(uint64_t z) {  /* world.rs:397-402 */
    z = z + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static inline double xs_next(uint64_t* st) {  /* world.rs:386-391 */
    uint64_t x = *st;
    x ^= x << 13;
    x ^= x >> 7;
    x ^= x << 17;
    *st = x;
    return (double)(x >> 11) / 9007199254740992.0;
}

static inline double gs(double u1, double u2) {  /* world.rs:393-395 */
    double s, c;
    mqr_sincos2pi(u2, &s, &c);
    return sqrt(-2.0 * mqr_log(u1 > 1e-300 ? u1 : 1e-300)) * c;
}

/* ------------------------------------------------------------------ per-batch / per-job constants */

typedef struct {
    double dt, v_rf, w_rf, h, inv_h;   /* inv_h unused by the f64 path: x / h is divided */
    double z_return, z_exit, crash_z0, crash_z1;
    double lim[3];
    double a;
    uint32_t max_steps;
    int nearest, legacy_coll;
} bconst;

typedef struct {
    double qmdt, v_ac, w_ac, nsd, s_gas, mr, floor_v, mfp_mean, s_ion, m;
    int use_ac, tab;
} jconst;

uint32_t mqr_max_steps(const mqr_batch* b) {
    double s = floor(b->t_max / b->dt + 0.5);   /* (T_MAX / DT).round(), world.rs:360 */
    if (!(s >= 0)) return 0;
    if (s > 4294967295.0) return 4294967295u;
    return (uint32_t)s;
}

static void make_bconst(const mqr_grid* g, const mqr_batch* b, bconst* c) {
    c->dt = b->dt;
    c->v_rf = b->v_rf;
    c->w_rf = b->f_rf * b->dt;
    c->h = g->h;
    c->inv_h = 1.0 / g->h;
    if (b->legacy_criteria) {   /* channel.rs:402-406 */
        c->z_return = 1.0e-3;
        c->z_exit = 23.7e-3;
        c->crash_z0 = b->layers_mm[0] * 1e-3;
        c->crash_z1 = b->layers_mm[1] * 1e-3;
    } else {
        c->z_return = 0.5e-3;
        c->z_exit = b->layers_mm[4] * 1e-3;
        c->crash_z0 = -1.0;
        c->crash_z1 = 1.0;
    }
    c->lim[0] = (double)(g->nx - 1) * g->h;
    c->lim[1] = (double)(g->ny - 1) * g->h;
    c->lim[2] = (double)(g->nz - 1) * g->h;
    c->a = b->axis_mm * 1e-3;
    c->max_steps = mqr_max_steps(b);
    c->nearest = b->legacy_fields;
    c->legacy_coll = b->legacy_collisions;
}

static double legacy_mfp_mean(const mqr_job* j, const mqr_batch* b) {  /* channel.rs:376-381 */
    double p_torr = b->pressure_pa / 133.322 + 1e-10;
    double np = 2.68e5 * (p_torr / 760.0);
    double m = j->mass;
    double ccs_he = 2.81e-9 * m * m * m - 3.55e-5 * m * m + 0.232 * m + 41.91;
    double ccs = ccs_he * 10.0 * sqrt(j->z);
    return 1.0 / (np * ccs);
}

static void make_jconst(const mqr_job* j, const mqr_batch* b, jconst* c) {
    double m = j->mass * AMU, mg = 28.0 * AMU;
    double qm = j->z * QE / m;
    double n_gas = b->pressure_pa / (KB * b->temp_k);
    double s_gas = sqrt(KB * b->temp_k / mg);
    double qk = b->legacy_force ? 0.5 * qm : qm;   /* channel.rs:419 */
    c->qmdt = qk * b->dt;
    c->v_ac = j->v_ac;
    c->w_ac = j->f_ac * b->dt;
    c->nsd = (n_gas * (j->ccs_n2 * 1e-20)) * b->dt;   /* cfg.ngas * sp.sig * dt, world.rs:501 */
    c->s_gas = s_gas;
    c->mr = mg / (m + mg);
    c->floor_v = b->legacy_collisions ? sqrt(2.0 * 0.035 * 1.6e-19 / (j->mass * 1.66e-27)) : -1.0;
    c->mfp_mean = legacy_mfp_mean(j, b);
    c->s_ion = sqrt(KB * b->temp_k / m);
    c->m = m;
    c->use_ac = j->v_ac != 0.0;
    c->tab = 0;
}

/* ------------------------------------------------------------------ phase tables (Clock::fill) */

#define TAB_CAP (1u << 20)

typedef struct {
    double w;        /* cycles per step */
    uint32_t len;
    double* sc;      /* [2*n] = sin, [2*n+1] = cos of 2 pi frac(n w) */
} table;

static inline void phase_at(double w, uint32_t n, double* s, double* c) {
    double p = (double)n * w;
    mqr_sincos2pi(p - floor(p), s, c);
}

static void table_fill(table* t, double w, uint32_t len) {
    t->w = w;
    t->len = len;
    t->sc = (double*)malloc(sizeof(double) * 2 * (size_t)(len ? len : 1));
    for (uint32_t n = 0; n < len; ++n) phase_at(w, n, &t->sc[2 * n], &t->sc[2 * n + 1]);
}

static inline void table_get(const table* t, uint32_t n, double* s, double* c) {
    if (n < t->len) { *s = t->sc[2 * n]; *c = t->sc[2 * n + 1]; }
    else phase_at(t->w, n, s, c);
}

/* ------------------------------------------------------------------ injection */

static void inject_one(const mqr_batch* b, const bconst* bc, const jconst* jc, const mqr_job* j,
                       uint64_t seed, double* pos, double* vel, double* ph_rf, double* ph_ac,
                       int32_t* leg, uint64_t* rng_out) {
    uint64_t st = seed | 1ull;    /* Ion::inject, world.rs:408 */
    const double a = bc->a, zi = b->z_inject_mm * 1e-3;
    if (b->legacy_injection || b->launch == 1) {   /* chsim legacy launch, channel.rs:350-355 */
        double kin = 0.1 * (0.75 + 0.75 * xs_next(&st)) * j->z;
        double vin = sqrt(2.0 * kin * QE / jc->m);
        double ang = (-10.0 + 20.0 * xs_next(&st)) * (0x1.921fb54442d18p+1 / 180.0);
        double sa = sin_k(ang), ca = cos_k(ang);
        double vx = 0.707 * vin * sa;
        pos[0] = a; pos[1] = a; pos[2] = zi;
        vel[0] = vx; vel[1] = vx; vel[2] = vin * ca;
    } else {
        if (b->launch == 2) {   /* Gaussian spot about the axis (sigma per transverse axis) */
            double sg = b->sigma_mm * 1e-3;
            double u1 = xs_next(&st), u2 = xs_next(&st);
            pos[0] = a + sg * gs(u1, u2);
            u1 = xs_next(&st); u2 = xs_next(&st);
            pos[1] = a + sg * gs(u1, u2);
        } else {                /* effusive disc, world.rs:410-412 */
            double r = b->r_inject_mm * 1e-3 * sqrt(xs_next(&st));
            double s, c;
            mqr_sincos2pi(xs_next(&st), &s, &c);
            pos[0] = a + r * c;
            pos[1] = a + r * s;
        }
        pos[2] = zi;
        double u1 = xs_next(&st), u2 = xs_next(&st);
        vel[0] = jc->s_ion * gs(u1, u2);
        u1 = xs_next(&st); u2 = xs_next(&st);
        vel[1] = jc->s_ion * gs(u1, u2);
        u1 = xs_next(&st);
        vel[2] = jc->s_ion * sqrt(-2.0 * mqr_log(u1 > 1e-300 ? u1 : 1e-300));
    }
    *ph_ac = xs_next(&st);           /* world.rs:414 */
    double prf = xs_next(&st);       /* world.rs:415-416 */
    *ph_rf = b->rf_phase0 ? 0.0 : prf;
    /* first legacy free path has an extra /10 (channel.rs:365-366) */
    double u = xs_next(&st);
    double first = -mqr_log(u > 1e-7 ? u : 1e-7) * jc->mfp_mean / 10.0;
    double vmag = sqrt(vel[0] * vel[0] + vel[1] * vel[1] + vel[2] * vel[2]);
    double s0 = floor(first / vmag / bc->dt) + 1.0;
    *leg = !(s0 < 2147483647.0) ? 2147483647 : (int32_t)s0;
    *rng_out = st | 1ull;
}

int mqr_inject(const mqr_batch* b, const mqr_job* jobs, size_t njobs, mqr_ions* io, size_t n) {
    if (!b || !jobs || !io || njobs == 0) return -1;
    size_t tot = 0;
    for (size_t k = 0; k < njobs; ++k) tot += jobs[k].n;
    if (tot != n) return -1;
    mqr_grid dummy = {3, 3, 3, 1e-3, 0, 0, 0};
    bconst bc;
    make_bconst(&dummy, b, &bc);
    size_t i = 0;
    for (size_t k = 0; k < njobs; ++k) {
        jconst jc;
        make_jconst(&jobs[k], b, &jc);
        for (uint64_t q = 0; q < jobs[k].n; ++q, ++i) {
            uint64_t seed = mqr_splitmix(jobs[k].seed + q * 0x9E37ull);   /* validate.rs:28 */
            double pos[3], vel[3];
            inject_one(b, &bc, &jc, &jobs[k], seed, pos, vel, &io->ph_rf[i], &io->ph_ac[i], &io->leg[i], &io->rng[i]);
            io->x[i] = pos[0]; io->y[i] = pos[1]; io->z[i] = pos[2];
            io->vx[i] = vel[0]; io->vy[i] = vel[1]; io->vz[i] = vel[2];
            io->steps[i] = 0; io->ncoll[i] = 0; io->status[i] = 0; io->jid[i] = (uint32_t)k;
        }
    }
    return 0;
}

/* ------------------------------------------------------------------ fields and tests */

static inline size_t cell_lo(double g, int n) {   /* (g.max(0.0) as usize).min(n - 2) */
    if (!(g > 0.0)) return 0;
    if (g >= (double)(n - 2)) return (size_t)(n - 2);
    return (size_t)g;
}

/* World::fields_at (world.rs:265-288); nearest = chsim legacy fields (t = 0, channel.metal:60) */
static inline void fields_at(const mqr_grid* g, int nearest, const double x[3], double er[3],
                             double ea[3], double ed[3]) {
    const double h = g->h;
    double gg[3] = {x[0] / h, x[1] / h, x[2] / h};
    size_t i = cell_lo(gg[0], g->nx), j = cell_lo(gg[1], g->ny), k = cell_lo(gg[2], g->nz);
    double tx = gg[0] - (double)i, ty = gg[1] - (double)j, tz = gg[2] - (double)k;
    if (nearest) { tx = 0.0; ty = 0.0; tz = 0.0; }
    for (int d = 0; d < 3; ++d) { er[d] = 0.0; ea[d] = 0.0; ed[d] = 0.0; }
    const size_t nx = (size_t)g->nx, ny = (size_t)g->ny;
    for (int di = 0; di < 2; ++di) {
        double wx = di ? tx : 1.0 - tx;
        for (int dj = 0; dj < 2; ++dj) {
            double wy = dj ? ty : 1.0 - ty;
            for (int dk = 0; dk < 2; ++dk) {
                double wz = dk ? tz : 1.0 - tz;
                size_t q = (i + di) + nx * ((j + dj) + ny * (k + dk));
                double w = wx * wy * wz;
                const float* r = g->rf4 + 4 * q;
                const float* a = g->ac4 + 4 * q;
                const float* c = g->dc4 + 4 * q;
                for (int d = 0; d < 3; ++d) {
                    er[d] += w * (double)r[d];
                    ea[d] += w * (double)a[d];
                    ed[d] += w * (double)c[d];
                }
            }
        }
    }
}

static inline size_t node_round(double g, int n) {   /* ((x / h).round() as usize).min(n - 1) */
    double r = round(g);
    if (!(r > 0.0)) return 0;
    if (r >= (double)(n - 1)) return (size_t)(n - 1);
    return (size_t)r;
}

/* ------------------------------------------------------------------ one ion */

typedef struct {
    const mqr_grid* g;
    const mqr_batch* b;
    const bconst* bc;
    const jconst* jc;      /* per job */
    const table* rf;
    const table* ac;       /* per tone */
    mqr_ions* io;
} ctx_t;

/* advance ion i by at most max_more steps (advance_with_field, world.rs:498-536, with the
 * chsim switches); returns executed steps */
static uint32_t advance_ion(const ctx_t* C, size_t i, uint32_t max_more) {
    mqr_ions* io = C->io;
    if (io->status[i] != 0) return 0;
    const bconst* bc = C->bc;
    const jconst* jc = &C->jc[io->jid[i]];
    const table* tac = &C->ac[jc->tab];
    double x[3] = {io->x[i], io->y[i], io->z[i]};
    double v[3] = {io->vx[i], io->vy[i], io->vz[i]};
    uint64_t rng = io->rng[i];
    uint32_t age = io->steps[i], ncoll = io->ncoll[i];
    int32_t leg = io->leg[i];
    int32_t status = 0;
    double rs, rc, as_, ac;
    mqr_sincos2pi(io->ph_rf[i], &rs, &rc);
    mqr_sincos2pi(io->ph_ac[i], &as_, &ac);
    const double dt = bc->dt, qmdt = jc->qmdt;
    uint32_t done = 0;
    while (done < max_more) {
        double S, Cc, Sa = 0.0, Ca = 0.0;
        table_get(C->rf, age, &S, &Cc);
        double srf = bc->v_rf * (S * rc + Cc * rs);
        double sac = 0.0;
        if (jc->use_ac) {
            table_get(tac, age, &Sa, &Ca);
            sac = jc->v_ac * (Sa * ac + Ca * as_);
        }
        double er[3], ea[3], ed[3];
        fields_at(C->g, bc->nearest, x, er, ea, ed);
        for (int d = 0; d < 3; ++d) {
            v[d] += qmdt * (srf * er[d] + sac * ea[d] + ed[d]);
            x[d] += v[d] * dt;
        }
        age += 1;
        done += 1;
        if (!bc->legacy_coll) {   /* collide, world.rs:473-488 */
            double vm = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
            double bound = vm + 6.0 * jc->s_gas;
            if (xs_next(&rng) < jc->nsd * bound) {
                double vg[3];
                for (int d = 0; d < 3; ++d) {
                    double u1 = xs_next(&rng), u2 = xs_next(&rng);
                    vg[d] = jc->s_gas * gs(u1, u2);
                }
                double gv[3] = {v[0] - vg[0], v[1] - vg[1], v[2] - vg[2]};
                double gl = sqrt(gv[0] * gv[0] + gv[1] * gv[1] + gv[2] * gv[2]);
                if (xs_next(&rng) * bound < gl) {
                    double c = 2.0 * xs_next(&rng) - 1.0;
                    double sp, cp;
                    mqr_sincos2pi(xs_next(&rng), &sp, &cp);
                    double omc = 1.0 - c * c;
                    double sn = sqrt(omc > 0.0 ? omc : 0.0);
                    double nn[3] = {sn * cp, sn * sp, c};
                    for (int d = 0; d < 3; ++d) v[d] = v[d] - jc->mr * gv[d] + jc->mr * gl * nn[d];
                    ncoll += 1;
                }
            }
        } else {                  /* legacy stationary-gas collision, channel.metal:100-113 */
            leg -= 1;
            if (leg <= 0) {
                double vm = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
                if (vm > jc->floor_v) {
                    double c = 2.0 * xs_next(&rng) - 1.0;
                    double sp, cp;
                    mqr_sincos2pi(xs_next(&rng), &sp, &cp);
                    double omc = 1.0 - c * c;
                    double sn = sqrt(omc > 0.0 ? omc : 0.0);
                    double dd[3] = {sn * cp, sn * sp, c};
                    double k1 = 1.0 - jc->mr, k2 = jc->mr * vm;
                    for (int d = 0; d < 3; ++d) v[d] = v[d] * k1 + k2 * dd[d];
                    ncoll += 1;
                }
                double u = xs_next(&rng);
                double mfp = -mqr_log(u > 1e-7 ? u : 1e-7) * jc->mfp_mean;
                double vn = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
                double st = floor(mfp / (vn > 1e-3 ? vn : 1e-3) / dt);
                if (st < 1.0) st = 1.0;
                leg = !(st < 2147483647.0) ? 2147483647 : (int32_t)st;
            }
        }
        /* termination tests: exit, return (world.rs:524-525), box, conductor (world.rs:309-313
           with chsim's crash window), timeout */
        if (x[2] > bc->z_exit) { status = 3; break; }
        if (x[2] < bc->z_return) { status = 2; break; }
        if (x[0] < 0.0 || x[1] < 0.0 || x[2] < 0.0 || x[0] > bc->lim[0] || x[1] > bc->lim[1] || x[2] > bc->lim[2]) { status = 4; break; }
        if (x[2] > bc->crash_z0 && x[2] < bc->crash_z1) {
            const mqr_grid* g = C->g;
            size_t ni = node_round(x[0] / g->h, g->nx), nj = node_round(x[1] / g->h, g->ny), nk = node_round(x[2] / g->h, g->nz);
            size_t q = ni + (size_t)g->nx * (nj + (size_t)g->ny * nk);
            if (g->rf4[4 * q + 3] > 0.5f) { status = 1; break; }
        }
        if (age >= bc->max_steps) { status = 5; break; }
    }
    io->x[i] = x[0]; io->y[i] = x[1]; io->z[i] = x[2];
    io->vx[i] = v[0]; io->vy[i] = v[1]; io->vz[i] = v[2];
    io->rng[i] = rng; io->steps[i] = age; io->ncoll[i] = ncoll; io->leg[i] = leg; io->status[i] = status;
    return done;
}

/* ------------------------------------------------------------------ threads (advance_all) */

typedef struct {
    const ctx_t* C;
    size_t i0, i1;
    uint32_t max_more;
    size_t next;             /* shared chunk counter */
    uint64_t steps;          /* guarded by lock */
    pthread_mutex_t lock;
} work_t;

static void* worker(void* arg) {
    work_t* W = (work_t*)arg;
    uint64_t local = 0;
    for (;;) {
        size_t c = __atomic_fetch_add(&W->next, 16, __ATOMIC_RELAXED);
        size_t a = W->i0 + c;
        if (a >= W->i1) break;
        size_t e = a + 16 < W->i1 ? a + 16 : W->i1;
        for (size_t i = a; i < e; ++i) local += advance_ion(W->C, i, W->max_more);
    }
    pthread_mutex_lock(&W->lock);
    W->steps += local;
    pthread_mutex_unlock(&W->lock);
    return NULL;
}

static int nthreads_default(void) {
    long n = sysconf(_SC_NPROCESSORS_ONLN);
    return n > 0 ? (int)n : 1;
}

int mqr_run_range(const mqr_grid* g, const mqr_batch* b, const mqr_job* jobs, size_t njobs,
                  mqr_ions* io, size_t i0, size_t i1, uint32_t max_more, int32_t threads,
                  uint64_t* steps_out) {
    if (!g || !b || !jobs || !io || njobs == 0 || i1 < i0 || g->nx < 2 || g->ny < 2 || g->nz < 2) return -1;
    bconst bc;
    make_bconst(g, b, &bc);
    jconst* jc = (jconst*)calloc(njobs, sizeof(jconst));
    table* tabs = (table*)calloc(njobs, sizeof(table));
    if (!jc || !tabs) { free(jc); free(tabs); return -2; }
    uint32_t tlen = bc.max_steps < TAB_CAP ? bc.max_steps : TAB_CAP;
    size_t ntab = 0;
    for (size_t k = 0; k < njobs; ++k) {
        make_jconst(&jobs[k], b, &jc[k]);
        size_t t;
        for (t = 0; t < ntab; ++t) if (tabs[t].w == jc[k].w_ac) break;   /* one table per tone */
        if (t == ntab) { table_fill(&tabs[ntab], jc[k].w_ac, jc[k].use_ac ? tlen : 0); ++ntab; }
        else if (jc[k].use_ac && tabs[t].len == 0) { free(tabs[t].sc); table_fill(&tabs[t], jc[k].w_ac, tlen); }
        jc[k].tab = (int)t;
    }
    table rf;
    table_fill(&rf, bc.w_rf, tlen);
    ctx_t C = {g, b, &bc, jc, &rf, tabs, io};
    int nt = threads > 0 ? threads : nthreads_default();
    work_t W;
    W.C = &C; W.i0 = i0; W.i1 = i1; W.max_more = max_more; W.next = 0; W.steps = 0;
    pthread_mutex_init(&W.lock, NULL);
    pthread_t* th = (pthread_t*)calloc((size_t)nt, sizeof(pthread_t));
    int started = 0;
    for (int t = 1; t < nt; ++t) if (pthread_create(&th[t], NULL, worker, &W) == 0) ++started; else th[t] = 0;
    worker(&W);
    for (int t = 1; t < nt; ++t) if (th[t]) pthread_join(th[t], NULL);
    pthread_mutex_destroy(&W.lock);
    if (steps_out) *steps_out = W.steps;
    free(th);
    free(rf.sc);
    for (size_t t = 0; t < ntab; ++t) free(tabs[t].sc);
    free(tabs);
    free(jc);
    (void)started;
    return 0;
}

int mqr_run(const mqr_grid* g, const mqr_batch* b, const mqr_job* jobs, size_t njobs,
            mqr_ions* io, size_t n, int32_t threads, uint64_t* steps_out) {
    return mqr_run_range(g, b, jobs, njobs, io, 0, n, 0xFFFFFFFFu, threads, steps_out);
}

int mqr_summarize(const mqr_ions* io, size_t n, const mqr_batch* b, size_t njobs, mqr_outcome* out) {
    if (!io || !out || !b) return -1;
    memset(out, 0, sizeof(mqr_outcome) * njobs);
    /* sums of collisions and steps are kept as integers, so the means do not depend on ion order */
    uint64_t* acc = (uint64_t*)calloc(2 * (njobs ? njobs : 1), sizeof(uint64_t));
    if (!acc) return -2;
    for (size_t i = 0; i < n; ++i) {   /* channel.rs:496-506 */
        uint32_t j = io->jid[i];
        if (j >= njobs) { free(acc); return -1; }
        mqr_outcome* o = &out[j];
        o->n += 1;
        switch (io->status[i]) {
            case 1: o->crashed += 1; break;
            case 2: o->returned += 1; break;
            case 3: o->transmitted += 1; break;
            case 4: o->left += 1; break;
            default: o->timeout += 1; break;
        }
        acc[2 * j] += io->ncoll[i];
        acc[2 * j + 1] += io->steps[i];
    }
    for (size_t j = 0; j < njobs; ++j)
        if (out[j].n) {
            out[j].mean_coll = (double)acc[2 * j] / (double)out[j].n;
            out[j].mean_time = (double)acc[2 * j + 1] * b->dt / (double)out[j].n;
        }
    free(acc);
    return 0;
}


/* ------------------------------------------------------------------ independent form (validate.rs:49-94) */

/* one field of the grid by a separate trilinear pass (world.rs:112-131, tri_one): weights
   ((wx wy) wz) per corner, corners in i, j, k order */
static void tri_one(const mqr_grid* g, const float* f4, const double x[3], double e[3]) {
    const double gx = x[0] / g->h, gy = x[1] / g->h, gz = x[2] / g->h;
    const size_t i = cell_lo(gx, g->nx), j = cell_lo(gy, g->ny), k = cell_lo(gz, g->nz);
    const double tx = gx - (double)i, ty = gy - (double)j, tz = gz - (double)k;
    e[0] = e[1] = e[2] = 0.0;
    for (int di = 0; di < 2; ++di)
        for (int dj = 0; dj < 2; ++dj)
            for (int dk = 0; dk < 2; ++dk) {
                const double wx = di ? tx : 1.0 - tx, wy = dj ? ty : 1.0 - ty, wz = dk ? tz : 1.0 - tz;
                const size_t q = (i + di) + (size_t)g->nx * ((j + dj) + (size_t)g->ny * (k + dk));
                for (int d = 0; d < 3; ++d) e[d] += wx * wy * wz * (double)f4[4 * q + d];
            }
}

typedef struct {
    const mqr_grid* g;
    const mqr_indep* p;
    uint64_t i0, i1;
    mqr_counts c;
} indep_job;

static void* indep_worker(void* arg) {
    indep_job* J = (indep_job*)arg;
    const mqr_grid* g = J->g;
    const mqr_indep* P = J->p;
    const double m = P->mass * AMU, mg = 28.0 * AMU;
    const double qm = P->z * QE / m, s_ion = sqrt(KB * 300.0 / m), mr = mg / (m + mg), sig = P->ccs_n2 * 1e-20;
    const double ngas = P->pressure_pa / (KB * 300.0), s_gas = sqrt(KB * 300.0 / mg);
    const double a = P->axis_mm * 1e-3, dt = P->dt;
    const double lim[3] = {(double)(g->nx - 1) * g->h, (double)(g->ny - 1) * g->h, (double)(g->nz - 1) * g->h};
    for (uint64_t id = J->i0; id < J->i1; ++id) {
        uint64_t st = (id + 1) * 0x9E3779B97F4A7C15ull ^ P->seed;
        const double r = 2.0e-3 * sqrt(xs_next(&st));
        double sn, cs;
        mqr_sincos2pi(xs_next(&st), &sn, &cs);
        double x[3] = {a + r * cs, a + r * sn, 1.0e-3};
        double u1 = xs_next(&st), u2 = xs_next(&st);
        double v[3];
        v[0] = s_ion * gs(u1, u2);
        u1 = xs_next(&st); u2 = xs_next(&st);
        v[1] = s_ion * gs(u1, u2);
        u1 = xs_next(&st);
        v[2] = s_ion * sqrt(-2.0 * mqr_log(u1 > 1e-300 ? u1 : 1e-300));
        const double ph_ac = xs_next(&st);                  /* phases in turns */
        double ph_rf = xs_next(&st);
        if (P->rf_phase0) ph_rf = 0.0;
        double t = 0.0;
        uint64_t steps = 0;
        int out = 5;
        while (t < P->t_max) {
            /* sin(2 pi (f t + phase)): this library's turn-based sine, own time accumulator */
            double p = P->f_rf * t + ph_rf, s1, c1, s2, c2;
            mqr_sincos2pi(p - floor(p), &s1, &c1);
            p = P->f_ac * t + ph_ac;
            mqr_sincos2pi(p - floor(p), &s2, &c2);
            const double srf = s1 * P->v_rf, sac = s2 * P->v_ac;
            double er[3], ea[3], ed[3];
            tri_one(g, g->rf4, x, er);
            tri_one(g, g->ac4, x, ea);
            tri_one(g, g->dc4, x, ed);
            for (int d = 0; d < 3; ++d) {
                v[d] += qm * dt * (srf * er[d] + sac * ea[d] + ed[d]);
                x[d] += v[d] * dt;
            }
            t += dt;
            steps += 1;
            const double vm = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
            const double bound = vm + 6.0 * s_gas;
            if (xs_next(&st) < ngas * sig * dt * bound) {
                double vg[3];
                for (int d = 0; d < 3; ++d) {
                    u1 = xs_next(&st);
                    u2 = xs_next(&st);
                    vg[d] = s_gas * gs(u1, u2);
                }
                const double gv[3] = {v[0] - vg[0], v[1] - vg[1], v[2] - vg[2]};
                const double gl = sqrt(gv[0] * gv[0] + gv[1] * gv[1] + gv[2] * gv[2]);
                if (xs_next(&st) * bound < gl) {
                    const double c = 2.0 * xs_next(&st) - 1.0;
                    double sp, cp;
                    mqr_sincos2pi(xs_next(&st), &sp, &cp);
                    const double omc = 1.0 - c * c;
                    const double snn = sqrt(omc > 0.0 ? omc : 0.0);
                    const double nn[3] = {snn * cp, snn * sp, c};
                    for (int d = 0; d < 3; ++d) v[d] = v[d] - mr * gv[d] + mr * gl * nn[d];
                }
            }
            if (x[2] > P->z_exit) { out = 3; break; }
            if (x[2] < P->z_return) { out = 2; break; }
            int crash = x[0] < 0.0 || x[1] < 0.0 || x[2] < 0.0 || x[0] > lim[0] || x[1] > lim[1] || x[2] > lim[2];
            if (!crash) {
                const size_t q = node_round(x[0] / g->h, g->nx) +
                                 (size_t)g->nx * (node_round(x[1] / g->h, g->ny) + (size_t)g->ny * node_round(x[2] / g->h, g->nz));
                crash = g->rf4[4 * q + 3] > 0.5f;
            }
            if (crash) { out = 1; break; }
        }
        J->c.steps += steps;
        J->c.n += 1;
        if (out == 3) J->c.transmitted += 1;
        else if (out == 2) J->c.returned += 1;
        else if (out == 1) J->c.crashed += 1;
        else J->c.timeout += 1;
    }
    return NULL;
}

int mqr_run_independent(const mqr_grid* g, const mqr_indep* p, uint64_t n, int32_t threads, mqr_counts* out) {
    if (!g || !p || !out || !(p->dt > 0)) return -1;
    int nt = threads > 0 ? threads : nthreads_default();
    if ((uint64_t)nt > n) nt = n ? (int)n : 1;
    indep_job* jobs = (indep_job*)calloc((size_t)nt, sizeof(indep_job));
    pthread_t* th = (pthread_t*)calloc((size_t)nt, sizeof(pthread_t));
    if (!jobs || !th) { free(jobs); free(th); return -2; }
    for (int t = 0; t < nt; ++t) {
        jobs[t].g = g; jobs[t].p = p;
        jobs[t].i0 = n * (uint64_t)t / (uint64_t)nt;
        jobs[t].i1 = n * (uint64_t)(t + 1) / (uint64_t)nt;
    }
    for (int t = 1; t < nt; ++t) pthread_create(&th[t], NULL, indep_worker, &jobs[t]);
    indep_worker(&jobs[0]);
    for (int t = 1; t < nt; ++t) pthread_join(th[t], NULL);
    memset(out, 0, sizeof(*out));
    for (int t = 0; t < nt; ++t) {
        out->n += jobs[t].c.n; out->transmitted += jobs[t].c.transmitted; out->crashed += jobs[t].c.crashed;
        out->returned += jobs[t].c.returned; out->timeout += jobs[t].c.timeout; out->steps += jobs[t].c.steps;
    }
    free(jobs);
    free(th);
    return 0;
}
