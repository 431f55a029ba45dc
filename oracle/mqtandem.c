/*
 * mqtandem.c -- CPU oracle of the tandem transport (TEST INFRASTRUCTURE ONLY; mqtandem.h lists
 * the reference functions restated here).  Built with mqref.c into _ref/libmqref.so with
 * -ffp-contract=off.
 */
#define _GNU_SOURCE
#include "mqtandem.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include "mqref.h"

static const double AMU_ = 1.6605390666e-27;   /* world.rs:13-15 */
static const double QE_ = 1.602176634e-19;
static const double KB_ = 1.380649e-23;
static const double ZEXIT = 18.6e-3;            /* world.rs:21-22 */
static const double ZRET = 0.5e-3;

enum { FREE = 0, POST = 1, PLANE = 2, ENT = 3, EXT = 4 };
enum { SPLIT = 0, COMBINE = 10, LOST = 11, BACK = 12, DETECTED = 13 };
enum { C_ENT = 0, C_RET = 1, C_FWD = 2, C_REV = 3, C_OTHER = 4, C_RETRY = 5, C_REVERSE = 14, C_LOST = 15, C_CHARGE = 16 };

/* ------------------------------------------------------------------ geometry */

void mqt_as_built(mqt_cube* g) {   /* geometry.rs:47-57 */
    memset(g, 0, sizeof(*g));
    g->n = 10;
    g->d = 6.34;
    g->pitch = 8.30;
    g->height = g->d;
    g->t_pcb = 1.5;
    g->gap = (g->pitch - g->d) / 2.0;
    g->stem_r = 2.0;
    g->clear_r = g->d / 2.0;
    g->l_ext = 6.0;
    g->ap_r = 4.0;
    g->rod_clear_extra = 0.5;
    g->cap_gap = 2.0;
    g->cap_r = 12.0;
    g->ent_axis = 1; g->ent_side = 1; g->ent_cell[0] = 4; g->ent_cell[1] = 4;
    g->ext_axis = 2; g->ext_side = 1; g->ext_cell[0] = 4; g->ext_cell[1] = 4;
}

static double c0_(const mqt_cube* g) { return g->t_pcb + g->gap + g->d / 2.0; }
double mqt_size(const mqt_cube* g) { return 2.0 * c0_(g) + (double)(g->n - 1) * g->pitch; }
static double lat_(const mqt_cube* g, int i) { return c0_(g) + g->pitch * (double)i; }
static double ptd_(const mqt_cube* g) { return g->t_pcb + g->gap + g->height; }
static double hyp_(double u, double v) { return sqrt(u * u + v * v); }

static int post_valid_(const mqt_cube* g, int a, const int idx[3]) {   /* geometry.rs:81-86 */
    if (idx[a] != 0 && idx[a] != g->n - 1) return 0;
    for (int a2 = a + 1; a2 < 3; ++a2)
        if (idx[a2] == 0 || idx[a2] == g->n - 1) return 0;
    return 1;
}

int mqt_n_posts(const mqt_cube* g) {   /* geometry.rs:87-94 */
    int c = 0;
    for (int i = 0; i < g->n; ++i)
        for (int j = 0; j < g->n; ++j)
            for (int k = 0; k < g->n; ++k) {
                const int idx[3] = {i, j, k};
                if (post_valid_(g, 0, idx) || post_valid_(g, 1, idx) || post_valid_(g, 2, idx)) ++c;
            }
    return c;
}

typedef struct { int axis, side, cell[2]; } pspec;

static pspec port_(const mqt_cube* g, int index) {   /* geometry.rs:114-117 */
    pspec p = {g->ext_axis, g->ext_side, {g->ext_cell[0], g->ext_cell[1]}};
    if (g->array) { p.cell[0] = 2 + 2 * (index % 3); p.cell[1] = 2 + 2 * (index / 3); }
    return p;
}

static void axis_xy_(const mqt_cube* g, const pspec* p, double* cb, double* cc) {   /* geometry.rs:109-113 */
    *cb = 0.5 * (lat_(g, p->cell[0]) + lat_(g, p->cell[0] + 1));
    *cc = 0.5 * (lat_(g, p->cell[1]) + lat_(g, p->cell[1] + 1));
}

static void posts_(const mqt_cube* g, const pspec* p, int out[4][3]) {   /* geometry.rs:96-108 */
    const int a = p->axis, b = (a + 1) % 3, c = (a + 2) % 3;
    int m = 0;
    for (int db = 0; db < 2; ++db)
        for (int dc = 0; dc < 2; ++dc, ++m) {
            out[m][a] = p->side == 0 ? 0 : g->n - 1;
            out[m][b] = p->cell[0] + db;
            out[m][c] = p->cell[1] + dc;
        }
}

static int round_idx_(double v, int hi) {   /* (v.round().clamp(0, hi)) as usize, NaN -> 0 */
    const double r = round(v);
    if (!(r > 0.0)) return 0;
    return r < (double)hi ? (int)r : hi;
}

int mqt_nearest_port(const mqt_cube* g, double x, double y) {   /* geometry.rs:118-125 */
    if (!g->array) return 0;
    const double first = (lat_(g, 2) + lat_(g, 3)) / 2.0;
    return round_idx_((x - first) / (2.0 * g->pitch), 2) + 3 * round_idx_((y - first) / (2.0 * g->pitch), 2);
}

void mqt_port_axis(const mqt_cube* g, int index, double xy[2]) {
    pspec p;
    if (index < 0) { p.axis = g->ent_axis; p.side = g->ent_side; p.cell[0] = g->ent_cell[0]; p.cell[1] = g->ent_cell[1]; }
    else p = port_(g, index);
    axis_xy_(g, &p, &xy[0], &xy[1]);
}

int mqt_classify(const mqt_cube* g, const double p[3], double gr, int32_t* sign) {   /* geometry.rs:136-205 */
    const double l = mqt_size(g), hd = g->d / 2.0;
    const int n = g->n;
    int fid = FREE, fsg = 0, plane = 0;
    int inside = 1;
    for (int a = 0; a < 3; ++a)
        if (!(p[a] >= -1e-12 && p[a] <= l + 1e-12)) inside = 0;
    for (int a = 0; a < 3; ++a) {
        const int b = (a + 1) % 3, c = (a + 2) % 3;
        for (int side = 0; side < 2; ++side) {
            const double u = side == 0 ? p[a] : l - p[a];
            int pid = 0;
            pspec ps = {0, 0, {0, 0}};
            if (g->ent_axis == a && g->ent_side == side) {
                pid = ENT;
                ps.axis = g->ent_axis; ps.side = g->ent_side; ps.cell[0] = g->ent_cell[0]; ps.cell[1] = g->ent_cell[1];
            } else if (g->ext_axis == a && g->ext_side == side) {
                pid = EXT;
                ps = port_(g, mqt_nearest_port(g, p[b], p[c]));
            }
            if (u < 0.0 || (pid && u < 0.0 + 1e-12)) {   /* outside the wall: port rods and end cap */
                if (pid) {
                    if (u <= -(g->l_ext + g->cap_gap)) {
                        double cb, cc;
                        axis_xy_(g, &ps, &cb, &cc);
                        if (hyp_(p[b] - cb, p[c] - cc) < g->cap_r) { *sign = 0; return pid; }
                    }
                    if (u >= -(g->l_ext + gr)) {
                        int pp[4][3];
                        posts_(g, &ps, pp);
                        for (int m = 0; m < 4; ++m)
                            if (hyp_(p[b] - lat_(g, pp[m][b]), p[c] - lat_(g, pp[m][c])) < hd + gr) {
                                *sign = (pp[m][0] + pp[m][1] + pp[m][2]) % 2 == 0 ? 1 : -1;
                                return pid;
                            }
                    }
                }
                continue;
            }
            if (!inside || u > ptd_(g) + gr) continue;
            int idx[3];
            idx[a] = side == 0 ? 0 : n - 1;
            idx[b] = round_idx_((p[b] - c0_(g)) / g->pitch, n - 1);
            idx[c] = round_idx_((p[c] - c0_(g)) / g->pitch, n - 1);
            const int valid = post_valid_(g, a, idx);
            const double dd = hyp_(p[b] - lat_(g, idx[b]), p[c] - lat_(g, idx[c]));
            const int sg = (idx[0] + idx[1] + idx[2]) % 2 == 0 ? 1 : -1;
            int rod = 0, aperture = 0;
            if (pid) {
                if (valid) {
                    int pp[4][3];
                    posts_(g, &ps, pp);
                    for (int m = 0; m < 4; ++m)
                        if (pp[m][0] == idx[0] && pp[m][1] == idx[1] && pp[m][2] == idx[2]) rod = pid;
                }
                double cb, cc;
                axis_xy_(g, &ps, &cb, &cc);
                if (hyp_(p[b] - cb, p[c] - cc) < g->ap_r - gr) aperture = 1;
            }
            if (rod && u <= ptd_(g) + gr && dd < hd + gr) { *sign = sg; return rod; }
            if (u <= g->t_pcb + gr) {
                const double hole = rod ? hd + g->rod_clear_extra : g->clear_r;
                if (!(aperture || (valid && dd < hole - gr))) plane = 1;
            }
            if (valid && !rod) {
                if (u <= g->t_pcb + g->gap + gr && dd < g->stem_r + gr) { fid = POST; fsg = sg; }
                if (u >= g->t_pcb + g->gap - gr && u <= ptd_(g) + gr && dd < hd + gr) { fid = POST; fsg = sg; }
            }
        }
    }
    if (fid != FREE) { *sign = fsg; return fid; }
    *sign = 0;
    return plane ? PLANE : FREE;
}

/* ------------------------------------------------------------------ model set-up */

void mqt_layout(const mqt_desc* d, double* seam, double* size, double mouths[18]) {   /* lib.rs:107-126 */
    const double sz = mqt_size(&d->cube) * 0.001;
    if (size) *size = sz;
    if (seam) *seam = sz - (ptd_(&d->cube) + d->ch_q1_start_mm - ZRET * 1000.0) * 0.001;
    if (mouths)
        for (int i = 0; i < 9; ++i) {
            double xy[2];
            mqt_port_axis(&d->cube, i, xy);
            mouths[2 * i] = xy[0] * 0.001;
            mouths[2 * i + 1] = xy[1] * 0.001;
        }
}

static double xs_(uint64_t* st) {   /* world.rs:385-391 */
    uint64_t x = *st;
    x ^= x << 13;
    x ^= x >> 7;
    x ^= x << 17;
    *st = x;
    return (double)(x >> 11) / 9007199254740992.0;
}

static double gs_(double u1, double u2) {   /* world.rs:393-395 */
    double s, c;
    mqr_sincos2pi(u2, &s, &c);
    return sqrt(-2.0 * mqr_log(u1 > 1e-300 ? u1 : 1e-300)) * c;
}

int mqt_inject(const mqt_desc* d, uint64_t seed, int mouth_start, mqt_tracks* tr, size_t n) {   /* lib.rs:131-160 */
    if (d->nspecies < 1 || d->nspecies > 5) return -1;
    double seam, size, mouths[18], ent[2];
    mqt_layout(d, &seam, &size, mouths);
    mqt_port_axis(&d->cube, -1, ent);
    double total = 0.0;
    for (int s = 0; s < d->nspecies; ++s) total += d->species[s].weight;
    for (size_t i = 0; i < n; ++i) {
        const uint64_t key = mqr_splitmix(seed + (uint64_t)i);
        double r = (double)(key >> 11) / 9007199254740992.0 * total;
        int sp = d->nspecies - 1;
        for (int s = 0; s < d->nspecies; ++s) {
            r -= d->species[s].weight;
            if (r <= 0.0) { sp = s; break; }
        }
        const double s_ion = sqrt(KB_ * d->temp_k / (d->species[sp].mass * AMU_));
        /* Ion::inject(splitmix(key), a = 0, ...) */
        uint64_t st = mqr_splitmix(key) | 1;
        const double rr = 2.0e-3 * sqrt(xs_(&st));
        double sn, cs;
        mqr_sincos2pi(xs_(&st), &sn, &cs);
        const double px = 0.0 + rr * cs, py = 0.0 + rr * sn;
        double u1 = xs_(&st), u2 = xs_(&st);
        const double vx = s_ion * gs_(u1, u2);
        u1 = xs_(&st);
        u2 = xs_(&st);
        const double vy = s_ion * gs_(u1, u2);
        u1 = xs_(&st);
        const double vz = s_ion * sqrt(-2.0 * mqr_log(u1 > 1e-300 ? u1 : 1e-300));
        xs_(&st);   /* AC phase */
        xs_(&st);   /* RF phase */
        tr->rng[i] = st | 1;
        tr->sp[i] = sp;
        tr->region[i] = SPLIT;
        tr->last[i] = -1;
        if (mouth_start) {
            tr->x[i] = mouths[2 * (i % 9)] + px;
            tr->y[i] = mouths[2 * (i % 9) + 1] + py;
            tr->z[i] = seam - 0.0001;
            tr->vx[i] = vx; tr->vy[i] = vy; tr->vz[i] = vz;
        } else {
            tr->x[i] = ent[1] * 0.001 + px * 0.1;
            tr->y[i] = size - 0.0001;
            tr->z[i] = ent[0] * 0.001 + py * 0.1;
            tr->vx[i] = vx; tr->vy[i] = -vz; tr->vz[i] = vy;
        }
    }
    return 0;
}

/* ------------------------------------------------------------------ routing */

void mqt_enter(mqt_tracks* tr, size_t k, int i, int from, double seam, const double c[2], double axis, uint32_t* cnt) {
    tr->x[k] += axis - c[0];
    tr->y[k] += axis - c[1];
    const double depth = tr->z[k] - seam;
    if (from == SPLIT) {
        tr->z[k] = ZRET + depth;
        cnt[C_ENT] += 1;
        if (tr->last[k] >= 0) {
            cnt[C_REV] += 1;
            cnt[C_RETRY + tr->last[k]] += 1;
            if (tr->last[k] != i) cnt[C_OTHER] += 1;
        }
    } else {
        tr->z[k] = ZEXIT - depth;
        tr->vz[k] *= -1.0;
        cnt[C_REVERSE] += 1;
    }
    tr->region[k] = 1 + i;
}

void mqt_leave(mqt_tracks* tr, size_t k, int i, double seam, const double c[2], double axis, uint32_t* cnt) {
    tr->x[k] += c[0] - axis;
    tr->y[k] += c[1] - axis;
    if (tr->z[k] < ZRET) {
        tr->z[k] = seam + tr->z[k] - ZRET;
        tr->region[k] = SPLIT;
        tr->last[k] = i;
        cnt[C_RET] += 1;
    } else {
        tr->z[k] = seam - (tr->z[k] - ZEXIT);
        tr->vz[k] *= -1.0;
        tr->region[k] = COMBINE;
        tr->last[k] = -1;
        cnt[C_FWD] += 1;
        cnt[C_CHARGE + tr->sp[k]] += 1;
    }
}

/* ------------------------------------------------------------------ fields and one step */

typedef struct {
    const mqt_desc* d;
    double seam, size, mouths[18], ent[2], axis, s_gas;
    double qmdt[8], mr[8], nsd[8];
    const double* drive;   /* [steps][10]: rf, ac[9] */
    mqt_tracks* tr;
    uint64_t steps;
} tctx;

static void cube_field_(const mqt_desc* d, const float* dc, const double x[3], double rf, double e[3]) {
    int c[3];
    double w[3];
    for (int a = 0; a < 3; ++a) {   /* fields.rs:89-96 */
        double f = (x[a] * 1000.0 - d->cube_lo_mm[a]) / d->cube_h_mm;
        const double hi = (double)(d->cube_dims[a] - 1) - 1e-9;
        if (f < 0.0) f = 0.0;
        else if (f > hi) f = hi;
        c[a] = f > 0.0 ? (int)floor(f) : 0;
        w[a] = f - (double)c[a];
    }
    e[0] = e[1] = e[2] = 0.0;
    const size_t nx = (size_t)d->cube_dims[0], ny = (size_t)d->cube_dims[1];
    for (int k = 0; k < 2; ++k)   /* lib.rs:70-88 */
        for (int j = 0; j < 2; ++j)
            for (int i = 0; i < 2; ++i) {
                const size_t q = (size_t)(c[0] + i) + nx * ((size_t)(c[1] + j) + ny * (size_t)(c[2] + k));
                const double wt = (i ? w[0] : 1.0 - w[0]) * (j ? w[1] : 1.0 - w[1]) * (k ? w[2] : 1.0 - w[2]);
                for (int a = 0; a < 3; ++a)
                    e[a] += wt * (rf * (double)d->cube_rf4[4 * q + a] + (double)dc[4 * q + a]);
            }
}

static int lo_cell_(double g, int n) {   /* (g.max(0.0) as usize).min(n - 2) */
    if (!(g > 0.0)) return 0;
    return g < (double)(n - 2) ? (int)g : n - 2;
}
static int near_node_(double g, int n) {   /* (g.round() as usize).min(n - 1) */
    const double r = round(g);
    if (!(r > 0.0)) return 0;
    return r < (double)(n - 1) ? (int)r : n - 1;
}

static void port_field_(const mqt_port* P, double gate_v, const double x[3], double rf, double ac, double e[3]) {
    const double h = P->h;
    const double g[3] = {x[0] / h, x[1] / h, x[2] / h};
    const int i0 = lo_cell_(g[0], P->dims[0]), j0 = lo_cell_(g[1], P->dims[1]), k0 = lo_cell_(g[2], P->dims[2]);
    const double tx = g[0] - (double)i0, ty = g[1] - (double)j0, tz = g[2] - (double)k0;
    const size_t nx = (size_t)P->dims[0], ny = (size_t)P->dims[1];
    double er[3] = {0, 0, 0}, ea[3] = {0, 0, 0}, ed[3] = {0, 0, 0};
    for (int di = 0; di < 2; ++di)   /* world.rs:265-288 */
        for (int dj = 0; dj < 2; ++dj)
            for (int dk = 0; dk < 2; ++dk) {
                const double wx = di ? tx : 1.0 - tx, wy = dj ? ty : 1.0 - ty, wz = dk ? tz : 1.0 - tz;
                const size_t q = (size_t)(i0 + di) + nx * ((size_t)(j0 + dj) + ny * (size_t)(k0 + dk));
                const double w = wx * wy * wz;
                for (int a = 0; a < 3; ++a) {
                    er[a] += w * (double)P->rf4[4 * q + a];
                    ea[a] += w * (double)P->ac4[4 * q + a];
                    ed[a] += w * (double)P->dc4[4 * q + a];
                }
            }
    double bias[3] = {0.0, 0.0, 0.0};
    if (P->tone_khz == 0.0)   /* gate_delta(x, 4 V), world.rs:291-302 */
        for (int i = 0; i < 2; ++i)
            for (int j = 0; j < 2; ++j)
                for (int k = 0; k < 2; ++k) {
                    const size_t q = (size_t)(i0 + i) + nx * ((size_t)(j0 + j) + ny * (size_t)(k0 + k));
                    const double w = gate_v * (i ? tx : 1.0 - tx) * (j ? ty : 1.0 - ty) * (k ? tz : 1.0 - tz);
                    for (int a = 0; a < 3; ++a) bias[a] += w * (double)P->gate4[4 * q + a];
                }
    for (int a = 0; a < 3; ++a) e[a] = rf * er[a] + ac * ea[a] + ed[a] + bias[a];
}

static int port_crash_(const mqt_port* P, const double x[3]) {   /* world.rs:309-314 */
    for (int a = 0; a < 3; ++a)
        if (x[a] < 0.0 || x[a] > (double)(P->dims[a] - 1) * P->h) return 1;
    const size_t q = (size_t)near_node_(x[0] / P->h, P->dims[0]) +
                     (size_t)P->dims[0] * ((size_t)near_node_(x[1] / P->h, P->dims[1]) +
                                           (size_t)P->dims[1] * (size_t)near_node_(x[2] / P->h, P->dims[2]));
    return P->rf4[4 * q + 3] > 0.5f;
}

static void collide_(double v[3], uint64_t* rng, double nsd, double mr, double s_gas) {   /* world.rs:473-488 */
    const double vm = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    const double bound = vm + 6.0 * s_gas;
    if (!(xs_(rng) < nsd * bound)) return;
    double vg[3];
    for (int a = 0; a < 3; ++a) {
        const double u1 = xs_(rng), u2 = xs_(rng);
        vg[a] = s_gas * gs_(u1, u2);
    }
    const double gv[3] = {v[0] - vg[0], v[1] - vg[1], v[2] - vg[2]};
    const double gl = sqrt(gv[0] * gv[0] + gv[1] * gv[1] + gv[2] * gv[2]);
    if (!(xs_(rng) * bound < gl)) return;
    const double c = 2.0 * xs_(rng) - 1.0;
    double sp, cp;
    mqr_sincos2pi(xs_(rng), &sp, &cp);
    const double omc = 1.0 - c * c;
    const double sn = sqrt(omc > 0.0 ? omc : 0.0);
    const double nn[3] = {sn * cp, sn * sp, c};
    for (int a = 0; a < 3; ++a) v[a] = v[a] - mr * gv[a] + mr * gl * nn[a];
}

static void run_track_(const tctx* C, size_t k, uint32_t* counts, uint64_t* nsteps) {
    const mqt_desc* d = C->d;
    mqt_tracks* tr = C->tr;
    const int sp = tr->sp[k];
    for (uint64_t s = 0; s < C->steps; ++s) {
        const int reg = tr->region[k];
        if (reg >= LOST) return;
        const double* dr = C->drive + 10 * s;
        double x[3] = {tr->x[k], tr->y[k], tr->z[k]}, v[3] = {tr->vx[k], tr->vy[k], tr->vz[k]}, e[3];
        if (reg == SPLIT || reg == COMBINE) {
            cube_field_(d, d->cube_dc4[reg == COMBINE], x, dr[0], e);
            nsteps[0] += 1;
        } else {
            port_field_(&d->port[reg - 1], d->gate_bias_v, x, dr[0], dr[reg], e);
            nsteps[d->port[reg - 1].tone_khz == 0.0 ? 2 : 1] += 1;
        }
        for (int a = 0; a < 3; ++a) {   /* transport_step, lib.rs:90-103 */
            v[a] += C->qmdt[sp] * e[a];
            x[a] += v[a] * d->dt;
        }
        collide_(v, &tr->rng[k], C->nsd[sp], C->mr[sp], C->s_gas);
        tr->x[k] = x[0]; tr->y[k] = x[1]; tr->z[k] = x[2];
        tr->vx[k] = v[0]; tr->vy[k] = v[1]; tr->vz[k] = v[2];
        if (reg == SPLIT || reg == COMBINE) {   /* lib.rs:212-253 */
            const double mm[3] = {x[0] * 1000.0, x[1] * 1000.0, x[2] * 1000.0};
            int32_t sg;
            if (mqt_classify(&d->cube, mm, 0.0, &sg) != FREE) { tr->region[k] = LOST; continue; }
            if (x[2] > C->seam) {
                const int i = mqt_nearest_port(&d->cube, mm[0], mm[1]);
                const double* c = &C->mouths[2 * i];
                if (hyp_(x[0] - c[0], x[1] - c[1]) < d->cube.ap_r * 0.001) {
                    mqt_enter(tr, k, i, reg, C->seam, c, C->axis, counts + (size_t)i * MQT_NC);
                    continue;
                }
                if (x[2] > C->size) { tr->region[k] = LOST; continue; }
            }
            if (x[1] > C->size && hyp_(mm[0] - C->ent[1], mm[2] - C->ent[0]) >= d->cube.ap_r) {
                tr->region[k] = LOST;
                continue;
            }
            if (x[1] > C->size + d->cube.l_ext * 0.001) tr->region[k] = reg == SPLIT ? BACK : DETECTED;
            else if (x[0] < 0.0 || x[1] < 0.0 || x[2] < 0.0 || x[0] > C->size) tr->region[k] = LOST;
        } else {   /* lib.rs:254-272 */
            const int i = reg - 1;
            if (port_crash_(&d->port[i], x)) {
                tr->region[k] = LOST;
                counts[(size_t)i * MQT_NC + C_LOST] += 1;
            } else if (x[2] < ZRET || x[2] > ZEXIT) {
                mqt_leave(tr, k, i, C->seam, &C->mouths[2 * i], C->axis, counts + (size_t)i * MQT_NC);
            }
        }
    }
}

typedef struct {
    const tctx* C;
    size_t i0, i1;
    uint32_t counts[9 * MQT_NC];
    uint64_t nsteps[3];
} tjob;

static void* tworker(void* arg) {
    tjob* j = (tjob*)arg;
    for (size_t k = j->i0; k < j->i1; ++k) run_track_(j->C, k, j->counts, j->nsteps);
    return NULL;
}

int mqt_advance(const mqt_desc* d, mqt_tracks* tr, size_t n, uint64_t step0, uint64_t steps, uint32_t* counts,
                int32_t threads, uint64_t* nsteps) {
    if (d->nspecies < 1 || d->nspecies > 5) return -1;
    for (size_t k = 0; k < n; ++k)
        if (tr->sp[k] < 0 || tr->sp[k] >= d->nspecies || tr->region[k] < 0 || tr->region[k] > DETECTED ||
            tr->last[k] < -1 || tr->last[k] > 8)
            return -1;
    tctx C;
    memset(&C, 0, sizeof(C));
    C.d = d;
    C.tr = tr;
    C.steps = steps;
    mqt_layout(d, &C.seam, &C.size, C.mouths);
    mqt_port_axis(&d->cube, -1, C.ent);
    C.axis = d->ch_axis_mm * 1e-3;
    const double mg = 28.0 * AMU_;   /* world.rs:27, 342-347, 358-362 */
    const double ngas = d->pressure_pa / (KB_ * d->temp_k);
    C.s_gas = sqrt(KB_ * d->temp_k / mg);
    for (int s = 0; s < d->nspecies; ++s) {
        const double m = d->species[s].mass * AMU_;
        C.qmdt[s] = d->species[s].z * QE_ / m * d->dt;
        C.mr[s] = mg / (m + mg);
        C.nsd[s] = ngas * (d->species[s].ccs * 1e-20) * d->dt;
    }
    double* drive = (double*)malloc(sizeof(double) * 10 * (steps ? steps : 1));
    if (!drive) return -2;
    for (uint64_t s = 0; s < steps; ++s) {   /* lib.rs:178-182 */
        const double t = (double)(step0 + s) * d->dt;
        double sn, cs, p = d->f_rf * t;
        mqr_sincos2pi(p - floor(p), &sn, &cs);
        drive[10 * s] = d->v_rf * sn;
        for (int i = 0; i < 9; ++i) {
            p = d->port[i].tone_khz * 1000.0 * t;
            mqr_sincos2pi(p - floor(p), &sn, &cs);
            drive[10 * s + 1 + i] = d->port[i].v_ac * sn;
        }
    }
    C.drive = drive;
    int nt = threads > 0 ? threads : (int)sysconf(_SC_NPROCESSORS_ONLN);
    if (nt < 1) nt = 1;
    if ((size_t)nt > n) nt = n ? (int)n : 1;
    tjob* jobs = (tjob*)calloc((size_t)nt, sizeof(tjob));
    pthread_t* th = (pthread_t*)calloc((size_t)nt, sizeof(pthread_t));
    if (!jobs || !th) { free(drive); free(jobs); free(th); return -2; }
    for (int t = 0; t < nt; ++t) {
        jobs[t].C = &C;
        jobs[t].i0 = n * (size_t)t / (size_t)nt;
        jobs[t].i1 = n * (size_t)(t + 1) / (size_t)nt;
    }
    for (int t = 1; t < nt; ++t) pthread_create(&th[t], NULL, tworker, &jobs[t]);
    tworker(&jobs[0]);
    for (int t = 1; t < nt; ++t) pthread_join(th[t], NULL);
    for (int t = 0; t < nt; ++t) {
        for (int q = 0; q < 9 * MQT_NC; ++q) counts[q] += jobs[t].counts[q];
        if (nsteps)
            for (int q = 0; q < 3; ++q) nsteps[q] += jobs[t].nsteps[q];
    }
    free(jobs);
    free(th);
    free(drive);
    return 0;
}
