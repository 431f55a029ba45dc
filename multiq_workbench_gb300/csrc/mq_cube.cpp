// Trap-cube set-up for the tandem transport: geometry helpers, the four cube field bases,
// fieldsolve's E-field stencils, the combined DC field, the tandem layout and the track
// launch.  CPU code, deterministic (-ffp-contract=off, per-plane work items).
//
// Reference: trapsim geometry/fields (simulation/trapsim/src/geometry.rs:47-205,
// fields.rs:28-96), fieldsolve efield_f32 (simulation/fieldsolve/src/field.rs:26-87),
// trapsim Model::new (simulation/trapsim/src/lib.rs:106-175).
#include <cmath>
#include <cstring>
#include <vector>

#include "mq_cube_geom.h"
#include "mq_phys.h"
#include "mq_pool.h"
#include "mq_tandem.h"

namespace {

// domain of the cube grid: the cube plus the port extensions (+ margin), geometry.rs:126-135
void domain(const mq_cube_geom& g, double margin, double lo[3], double hi[3]) {
    const double l = mqc::size(g);
    for (int a = 0; a < 3; ++a) { lo[a] = 0.0; hi[a] = l; }
    const int axes[2] = {g.ent_axis, g.ext_axis}, sides[2] = {g.ent_side, g.ext_side};
    for (int k = 0; k < 2; ++k) {
        if (sides[k] == 0) lo[axes[k]] = -(g.l_ext + margin);
        else hi[axes[k]] = l + g.l_ext + margin;
    }
}

}  // namespace

extern "C" {

void mq_cube_as_built(mq_cube_geom* g) {   // geometry.rs:47-57
    if (!g) return;
    std::memset(g, 0, sizeof(*g));
    const double d = 6.34, pitch = 8.30;
    g->n = 10; g->array = 0; g->d = d; g->pitch = pitch; g->height = d; g->t_pcb = 1.5; g->gap = (pitch - d) / 2.0;
    g->stem_r = 2.0; g->clear_r = d / 2.0; g->l_ext = 6.0; g->ap_r = 4.0; g->rod_clear_extra = 0.5; g->cap_gap = 2.0;
    g->cap_r = 12.0;
    g->ent_axis = 1; g->ent_side = 1; g->ent_cell[0] = 4; g->ent_cell[1] = 4;
    g->ext_axis = 2; g->ext_side = 1; g->ext_cell[0] = 4; g->ext_cell[1] = 4;
}

mq_status mq_cube_snap(const mq_cube_geom* g, double h_target, mq_cube_geom* out, double* h) {   // geometry.rs:66-73
    if (!g || !out || !h || !(h_target > 0)) return MQ_ERR_INVALID;
    double nh = std::round(g->pitch / (2.0 * h_target));
    if (nh < 1.0) nh = 1.0;
    const double hh = g->pitch / (2.0 * nh);
    *out = *g;
    out->t_pcb = std::round(g->t_pcb / hh) * hh;
    out->l_ext = std::round(g->l_ext / hh) * hh;
    *h = hh;
    return MQ_OK;
}

int32_t mq_cube_classify(const mq_cube_geom* g, const double p[3], double grow, int32_t* sign) {
    int s = 0;
    int id = mqc::classify(*g, p, grow, &s);
    if (sign) *sign = s;
    return id;
}

double mq_cube_size(const mq_cube_geom* g) { return g ? mqc::size(*g) : 0.0; }
double mq_cube_post_top_depth(const mq_cube_geom* g) { return g ? mqc::post_top_depth(*g) : 0.0; }
int32_t mq_cube_nearest_port(const mq_cube_geom* g, double x, double y) { return g ? mqc::nearest_port(*g, x, y) : -1; }

mq_status mq_cube_port_axis(const mq_cube_geom* g, int32_t index, double xy[2]) {
    if (!g || !xy) return MQ_ERR_INVALID;
    int p[4];
    if (index < 0) { p[0] = g->ent_axis; p[1] = g->ent_side; p[2] = g->ent_cell[0]; p[3] = g->ent_cell[1]; }
    else mqc::port(*g, index, p);
    int b, c;
    mqc::port_axis_xy(*g, p, &b, &c, &xy[0], &xy[1]);
    return MQ_OK;
}

mq_status mq_efield_fieldsolve(const double* phi, const uint8_t* mask, int32_t nx, int32_t ny, int32_t nz, double h,
                               float* e4) {
    if (!phi || !e4 || nx < 1 || ny < 1 || nz < 1 || !(h > 0)) return MQ_ERR_INVALID;
    const size_t sy = nx, sz = (size_t)nx * ny;
    auto elec = [&](size_t q) { return mask && mask[q] != 0; };
    // d phi / d axis at node q (index i of n along the axis, stride s), field.rs:26-57
    auto deriv = [&](size_t q, size_t s, int i, int n) -> double {
        const bool has_m = i > 0 && !elec(q - s);
        const bool has_p = i + 1 < n && !elec(q + s);
        if (has_m && has_p) return (phi[q + s] - phi[q - s]) / (2.0 * h);
        if (has_p) {
            if (i + 2 < n && !elec(q + 2 * s)) return (-3.0 * phi[q] + 4.0 * phi[q + s] - phi[q + 2 * s]) / (2.0 * h);
            return (phi[q + s] - phi[q]) / h;
        }
        if (has_m) {
            if (i >= 2 && !elec(q - 2 * s)) return (3.0 * phi[q] - 4.0 * phi[q - s] + phi[q - 2 * s]) / (2.0 * h);
            return (phi[q] - phi[q - s]) / h;
        }
        if (elec(q)) return 0.0;
        const bool lo = i > 0, hi = i + 1 < n;
        if (lo && hi) return (phi[q + s] - phi[q - s]) / (2.0 * h);
        if (hi) return (phi[q + s] - phi[q]) / h;
        if (lo) return (phi[q] - phi[q - s]) / h;
        return 0.0;
    };
    mq::Pool pool(0);
    pool.parallel_for(nz, [&](long k) {
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const size_t q = (size_t)i + sy * j + sz * k;
                e4[4 * q + 0] = (float)(-deriv(q, 1, i, nx));
                e4[4 * q + 1] = (float)(-deriv(q, sy, j, ny));
                e4[4 * q + 2] = (float)(-deriv(q, sz, (int)k, nz));
                e4[4 * q + 3] = (float)phi[q];
            }
    });
    return MQ_OK;
}

mq_status mq_cube_fields(const mq_cube_geom* g, double h_mm, double grow, double tol, int32_t threads, int32_t dims[3],
                         double lo_mm[3], float* rf4, float* wall4, float* ent4, float* ext4, mq_solve_stats stats[4]) {
    return mq_cube_fields_ex(g, h_mm, grow, tol, threads, -1, dims, lo_mm, rf4, wall4, ent4, ext4, stats);
}

mq_status mq_cube_fields_ex(const mq_cube_geom* g, double h_mm, double grow, double tol, int32_t threads, int32_t device,
                            int32_t dims[3], double lo_mm[3], float* rf4, float* wall4, float* ent4, float* ext4,
                            mq_solve_stats stats[4]) {
    if (!g || !dims || !lo_mm || !(h_mm > 0)) return MQ_ERR_INVALID;
    double lo[3], hi[3];
    domain(*g, g->cap_gap + 1.0, lo, hi);   // fields.rs:29
    int n[3];
    for (int a = 0; a < 3; ++a) {
        n[a] = (int)std::round((hi[a] - lo[a]) / h_mm) + 1;
        dims[a] = n[a];
        lo_mm[a] = lo[a];
    }
    if (!rf4 && !wall4 && !ent4 && !ext4) return MQ_OK;
    if (!rf4 || !wall4 || !ent4 || !ext4) return MQ_ERR_INVALID;
    const size_t len = (size_t)n[0] * n[1] * n[2];
    std::vector<uint8_t> id(len);
    std::vector<int8_t> sign(len);
    {
        mq::Pool pool(threads);
        pool.parallel_for(n[2], [&](long k) {   // fields.rs:38-44
            const double z = lo[2] + h_mm * (double)k;
            for (int j = 0; j < n[1]; ++j)
                for (int i = 0; i < n[0]; ++i) {
                    const double p[3] = {lo[0] + h_mm * (double)i, lo[1] + h_mm * (double)j, z};
                    int s = 0;
                    const size_t q = (size_t)i + (size_t)n[0] * ((size_t)j + (size_t)n[1] * k);
                    id[q] = (uint8_t)mqc::classify(*g, p, grow * h_mm, &s);
                    sign[q] = (int8_t)s;
                }
        });
    }
    std::vector<uint8_t> mask(len);
    std::vector<double> fixed(len), phi(len);
    float* outs[4] = {rf4, wall4, ent4, ext4};
    const double outer[4] = {0.0, 1.0, 0.0, 0.0};
    for (int b = 0; b < 4; ++b) {   // fields.rs:46-57: rf, wall, ent, ext problems
        for (size_t q = 0; q < len; ++q) {
            const int i = id[q];
            bool fx;
            double v = 0.0;
            if (b == 0) { fx = i == mqc::ID_POST || i == mqc::ID_ENT || i == mqc::ID_EXT || i == mqc::ID_PLANE;
                          v = (i == mqc::ID_PLANE) ? 0.0 : (double)sign[q]; }
            else { fx = i != mqc::ID_FREE;
                   v = (b == 1) ? (i == mqc::ID_PLANE ? 1.0 : 0.0) : (b == 2) ? (i == mqc::ID_ENT ? 1.0 : 0.0)
                                                                               : (i == mqc::ID_EXT ? 1.0 : 0.0); }
            mask[q] = fx ? 1 : 0;
            fixed[q] = fx ? v : 0.0;
        }
        mq_solve_stats st;
        mq_status s = device >= 0
                          ? mq_laplace_solve_device(n[0], n[1], n[2], mask.data(), fixed.data(), outer[b], tol, device, phi.data(), &st)
                          : mq_laplace_solve(n[0], n[1], n[2], mask.data(), fixed.data(), outer[b], tol, threads, phi.data(), &st);
        if (stats) stats[b] = st;
        if (s != MQ_OK) return s;   // assert!(st.converged), fields.rs:62
        s = mq_efield_fieldsolve(phi.data(), mask.data(), n[0], n[1], n[2], h_mm * 1e-3, outs[b]);
        if (s != MQ_OK) return s;
        if (b == 0)
            for (size_t q = 0; q < len; ++q) rf4[4 * q + 3] = (float)id[q];   // RF.w = electrode id (fields.rs:68)
    }
    return MQ_OK;
}

mq_status mq_cube_dc_combined(size_t n, const float* wall4, const float* ent4, const float* ext4, double u0, double uwall,
                              double q_in, double q_out, float* out4) {   // fields.rs:77-86
    if (!wall4 || !ent4 || !ext4 || !out4) return MQ_ERR_INVALID;
    const double w[3] = {uwall - u0, q_in - u0, q_out - u0};
    const float* B[3] = {wall4, ent4, ext4};
    for (size_t q = 0; q < n; ++q) {
        double e[4] = {0.0, 0.0, 0.0, 0.0};
        for (int b = 0; b < 3; ++b)
            for (int c = 0; c < 4; ++c) e[c] += w[b] * (double)B[b][4 * q + c];
        out4[4 * q + 0] = (float)e[0];
        out4[4 * q + 1] = (float)e[1];
        out4[4 * q + 2] = (float)e[2];
        out4[4 * q + 3] = (float)(e[3] + u0);
    }
    return MQ_OK;
}

mq_status mq_tandem_layout(const mq_tandem_desc* d, double* seam, double* size, double mouths[18]) {
    if (!d) return MQ_ERR_INVALID;
    const mq_cube_geom& g = d->cube;
    const double sz = mqc::size(g) * 0.001;
    // seam: where the channel's Q1 entrance plane meets the splitter (lib.rs:126)
    const double sm = sz - (mqc::post_top_depth(g) + d->ch_q1_start_mm - 0.5e-3 * 1000.0) * 0.001;
    if (seam) *seam = sm;
    if (size) *size = sz;
    if (mouths)
        for (int i = 0; i < 9; ++i) {
            int p[4], b, c;
            double xb, xc;
            mqc::port(g, i, p);
            mqc::port_axis_xy(g, p, &b, &c, &xb, &xc);
            mouths[2 * i] = xb * 0.001;
            mouths[2 * i + 1] = xc * 0.001;
        }
    return MQ_OK;
}

mq_status mq_tandem_inject(const mq_tandem_desc* d, uint64_t seed, int32_t mouth_start, mq_tracks* tr, size_t n) {
    if (!d || !tr || d->nspecies < 1 || d->nspecies > 5) return MQ_ERR_INVALID;
    double seam = 0, sz = 0, mouths[18];
    mq_tandem_layout(d, &seam, &sz, mouths);
    double total = 0.0;
    for (int s = 0; s < d->nspecies; ++s) total += d->species[s].weight;
    double ent[2];
    mq_cube_port_axis(&d->cube, -1, ent);   // entrance: (coordinate along z, coordinate along x)
    for (size_t i = 0; i < n; ++i) {        // lib.rs:131-160
        const uint64_t key = mqp::splitmix(seed + (uint64_t)i);
        double r = (double)(key >> 11) / 9007199254740992.0 * total;
        int sp = d->nspecies - 1;
        for (int s = 0; s < d->nspecies; ++s) {
            r -= d->species[s].weight;
            if (r <= 0.0) { sp = s; break; }
        }
        const double m = d->species[sp].mass * mqp::AMU;
        const double s_ion = sqrt(mqp::KB * d->temp_k / m);
        // Ion::inject with the axis at 0 (world.rs:407-422)
        uint64_t st = mqp::splitmix(key) | 1ull;
        const double rr = 2.0e-3 * sqrt(mqp::xs_next(&st));
        double sn, cs;
        mqp::sincos2pi(mqp::xs_next(&st), &sn, &cs);
        const double x0 = 0.0 + rr * cs, y0 = 0.0 + rr * sn;
        double u1 = mqp::xs_next(&st), u2 = mqp::xs_next(&st);
        const double vx = s_ion * mqp::gauss(u1, u2);
        u1 = mqp::xs_next(&st); u2 = mqp::xs_next(&st);
        const double vy = s_ion * mqp::gauss(u1, u2);
        u1 = mqp::xs_next(&st);
        const double vz = s_ion * sqrt(-2.0 * mqp::log_(u1 > 1e-300 ? u1 : 1e-300));
        (void)mqp::xs_next(&st);   // AC phase (unused: the tandem drives are global)
        (void)mqp::xs_next(&st);   // RF phase (0 for every ion)
        tr->rng[i] = st | 1ull;
        tr->sp[i] = sp;
        tr->region[i] = 0;
        tr->last[i] = -1;
        if (mouth_start) {
            const double* c = &mouths[2 * (i % 9)];
            tr->x[i] = c[0] + x0; tr->y[i] = c[1] + y0; tr->z[i] = seam - 0.0001;
            tr->vx[i] = vx; tr->vy[i] = vy; tr->vz[i] = vz;
        } else {
            tr->x[i] = ent[1] * 0.001 + x0 * 0.1; tr->y[i] = sz - 0.0001; tr->z[i] = ent[0] * 0.001 + y0 * 0.1;
            tr->vx[i] = vx; tr->vy[i] = -vz; tr->vz[i] = vy;
        }
    }
    return MQ_OK;
}

mq_status mq_tandem_frame(const mq_tracks* tr, size_t n, mq_tandem_frame_counts* o) {   // lib.rs:277-336
    if (!tr || !o) return MQ_ERR_INVALID;
    std::memset(o, 0, sizeof(*o));
    for (size_t i = 0; i < n; ++i) {
        const int r = tr->region[i];
        if (r == 0) o->split++;
        else if (r >= 1 && r <= 9) o->channel++;
        else if (r == 10) o->combine++;
        else if (r == 11) o->lost++;
        else if (r == 12) o->back++;
        else o->detected++;
    }
    return MQ_OK;
}

}  // extern "C"
