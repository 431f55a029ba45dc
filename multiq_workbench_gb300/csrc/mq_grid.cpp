// Field-grid set-up: channel geometry rasteriser, masked-Dirichlet Laplace solver,
// central-difference E field and combined DC field.  CPU code, deterministic on any
// host (built with -ffp-contract=off; reductions are summed per z-plane in plane order).
//
// Geometry follows chsim Geom (simulation/chsim/src/channel.rs:18-120); the solver meets
// fieldsolve's stopping rule (simulation/fieldsolve/src/lib.rs:156-166: scaled true
// max-norm residual of the 7-point operator <= tol, outer faces Dirichlet at outer_bc
// unless masked, initial guess outer_bc).  The solver itself is this project's own
// design: conjugate gradients preconditioned by one symmetric geometric V-cycle
// (red-black Gauss-Seidel, trilinear prolongation masked at fixed nodes, restriction
// = its transpose, re-discretised 7-point coarse operators).  CG makes it robust to
// thin plates and staircase electrodes without the Galerkin 27-point hierarchy the
// reference builds (simulation/fieldsolve/src/mg.rs:1-40).
#include "mq_grid.h"
#include "mq_levels.h"
#include "mq_pool.h"

#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

namespace {

// ------------------------------------------------------------------ geometry

struct Layers { double l[8]; };

Layers layers_of(const mq_geom* g) {
    Layers L;
    double l1 = g->q1_start, l2 = l1 + g->q1_len, l3 = l2 + g->gap, l4 = l3 + g->plate;
    double l5 = l4 + g->gap, l6 = l5 + g->q2_len, l7 = l6 + g->gap, l8 = l7 + g->plate;
    double v[8] = {l1, l2, l3, l4, l5, l6, l7, l8};
    for (int i = 0; i < 8; ++i) L.l[i] = v[i];
    return L;
}

int geom_nz(const mq_geom* g) { return (int)(layers_of(g).l[7] / g->h_mm + 1e-6); }
double geom_center(const mq_geom* g) { return g->coef * g->de / 2.0 + g->de / 2.0; }
double geom_axis(const mq_geom* g) { return (double)(g->n_xy / 2) * g->h_mm; }

// quadrant of (x, y) about the axis; -1 on an axis line (channel.rs:65-67)
inline int quad(double x, double y, double a) {
    if (x < a && y < a) return 0;
    if (x > a && y < a) return 1;
    if (x < a && y > a) return 2;
    if (x > a && y > a) return 3;
    return -1;
}

// rod membership test of channel.rs:70-79 (rod centre by quadrant and tilt mode)
bool rod_q(const mq_geom* g, double a, double c, double x, double y, double z, double zmid,
           int q, double sq, double d, bool q1) {
    double cx, cy;
    const double s2 = std::sqrt(2.0);
    if (g->tilt_mode == 0) {
        switch (q) {
            case 0: cx = a - c; cy = a - c + sq; break;
            case 1: cx = a + c; cy = a - c + sq; break;
            case 2: cx = a - c; cy = a + c - sq; break;
            default: cx = a + c; cy = a + c - sq; break;
        }
    } else if (g->tilt_mode == 2) {
        switch (q) {
            case 0: cx = a - c + sq / s2; cy = a - c + sq / s2; break;
            case 1: cx = a + c - sq / s2; cy = a - c + sq / s2; break;
            case 2: cx = a - c + sq / s2; cy = a + c - sq / s2; break;
            default: cx = a + c - sq / s2; cy = a + c - sq / s2; break;
        }
    } else {
        switch (q) {
            case 0: cx = a - c; cy = a - c; break;
            case 1: cx = a + c; cy = a - c; break;
            case 2: cx = a - c + sq; cy = a + c; break;
            default: cx = a + c - sq; cy = a + c; break;
        }
    }
    if (q1) {
        const double* m = g->mis[q];
        cx += m[0] + m[2] * (z - zmid);
        cy += m[1] + m[3] * (z - zmid);
    }
    double dx = x - cx, dy = y - cy;
    return std::sqrt(dx * dx + dy * dy) < d / 2.0 + g->grow * g->h_mm;
}

enum Kind { K_Q1 = 0, K_STEM3, K_PLATE, K_STEM5, K_Q2, K_STEM7, K_SLAB };
inline uint8_t code(int kind, int q) { return (uint8_t)(1 + kind * 4 + q); }

// Geom::classify (channel.rs:62-101): electrode code of node (i, j, k), 0 = free.
uint8_t classify(const mq_geom* g, const Layers& L, int i, int j, int k) {
    const double h = g->h_mm;
    const double x = i * h, y = j * h, z = k * h;
    const double a = geom_axis(g), c = geom_center(g);
    const double zmid = g->q1_start + g->q1_len / 2.0;
    const double eps = 1e-9;
    const double l1 = L.l[0], l2 = L.l[1], l3 = L.l[2], l4 = L.l[3], l5 = L.l[4], l6 = L.l[5],
                 l7 = L.l[6], l8 = L.l[7];
    if (z <= l1 + eps) return 0;
    if (z <= l2 + eps) {
        double sq = g->alpha * (l2 - z);
        int q = quad(x, y, a);
        return (q >= 0 && rod_q(g, a, c, x, y, z, zmid, q, sq, g->de, true)) ? code(K_Q1, q) : 0;
    }
    if (z <= l3 + eps) {
        int q = quad(x, y, a);
        return (q >= 0 && rod_q(g, a, c, x, y, z, zmid, q, 0.0, g->stem_d, false)) ? code(K_STEM3, q) : 0;
    }
    if (z <= l4 + eps) {
        double dx = x - a, dy = y - a;
        double r2 = dx * dx + dy * dy;
        double rh = g->hole_d / 2.0 - g->grow * g->h_mm;
        return r2 < rh * rh ? 0 : code(K_PLATE, 0);
    }
    if (z <= l5 + eps) {
        int q = quad(x, y, a);
        return (q >= 0 && rod_q(g, a, c, x, y, z, zmid, q, 0.0, g->stem_d, false)) ? code(K_STEM5, q) : 0;
    }
    if (z <= l6 + eps) {
        double sq = g->q2_flare_bug ? g->alpha * (l2 - z) : 0.0;
        int q = quad(x, y, a);
        return (q >= 0 && rod_q(g, a, c, x, y, z, zmid, q, sq, g->de, false)) ? code(K_Q2, q) : 0;
    }
    if (z <= l7 + eps) {
        int q = quad(x, y, a);
        return (q >= 0 && rod_q(g, a, c, x, y, z, zmid, q, 0.0, g->stem_d, false)) ? code(K_STEM7, q) : 0;
    }
    if (z <= l8 + eps) return code(K_SLAB, 0);
    return 0;
}

inline double rf_sign(int q) { return (q == 0 || q == 3) ? -1.0 : 1.0; }  // channel.rs:104
inline double ac_sign(int q) { return (q == 0 || q == 2) ? -1.0 : 1.0; }  // channel.rs:105

// basis_value (channel.rs:111-120) for an electrode code
double basis_value(int basis, uint8_t e, int ac_mode) {
    int kind = (e - 1) / 4, q = (e - 1) % 4;
    switch (basis) {
        case MQ_BASIS_RF:
            return (kind == K_Q1 || kind == K_STEM3 || kind == K_STEM5 || kind == K_Q2 || kind == K_STEM7) ? rf_sign(q) : 0.0;
        case MQ_BASIS_AC:
            if (kind == K_Q1 || kind == K_STEM3) return (ac_mode == 1 && q >= 2) ? 0.0 : ac_sign(q);
            return 0.0;
        case MQ_BASIS_DC_Q1: return (kind == K_Q1 || kind == K_STEM3) ? 1.0 : 0.0;
        case MQ_BASIS_DC_PLATE: return kind == K_PLATE ? 1.0 : 0.0;
        case MQ_BASIS_DC_DOWN: return (kind == K_STEM5 || kind == K_Q2 || kind == K_STEM7 || kind == K_SLAB) ? 1.0 : 0.0;
        default: return 0.0;
    }
}

// ------------------------------------------------------------------ multigrid-preconditioned CG

struct Level {
    int nx, ny, nz;
    std::vector<uint8_t> fix;   // 1 = Dirichlet (electrode, face, or coarse virtual node)
    std::vector<double> u, rhs, r;
    size_t n() const { return (size_t)nx * ny * nz; }
    size_t idx(int i, int j, int k) const { return (size_t)i + (size_t)nx * ((size_t)j + (size_t)ny * k); }
};

struct Solver {
    mq::Pool* pool;
    std::vector<Level> L;
    int nu = 2;            // smoothing sweeps (each a red + black half sweep)
    int coarse_sweeps = 60;

    // one Gauss-Seidel half sweep of colour `col` on S u = rhs (S = 6 - sum of neighbours)
    void gs_color(Level& lv, int col) {
        const int nx = lv.nx, ny = lv.ny;
        const size_t sy = nx, sz = (size_t)nx * ny;
        pool->parallel_for(lv.nz, [&](long k) {
            if (k == 0 || k == lv.nz - 1) return;
            for (int j = 1; j < ny - 1; ++j) {
                int i0 = 1 + ((1 + j + (int)k + col) & 1);
                size_t base = lv.idx(0, j, (int)k);
                for (int i = i0; i < nx - 1; i += 2) {
                    size_t q = base + i;
                    if (lv.fix[q]) continue;
                    double s = lv.u[q - 1] + lv.u[q + 1] + lv.u[q - sy] + lv.u[q + sy] + lv.u[q - sz] + lv.u[q + sz];
                    lv.u[q] = (lv.rhs[q] + s) / 6.0;
                }
            }
        });
    }
    // r = rhs - S u at free nodes, 0 elsewhere
    void residual(Level& lv) {
        const int nx = lv.nx, ny = lv.ny;
        const size_t sy = nx, sz = (size_t)nx * ny;
        pool->parallel_for(lv.nz, [&](long k) {
            for (int j = 0; j < ny; ++j) {
                size_t base = lv.idx(0, j, (int)k);
                for (int i = 0; i < nx; ++i) {
                    size_t q = base + i;
                    if (lv.fix[q]) { lv.r[q] = 0.0; continue; }
                    double s = lv.u[q - 1] + lv.u[q + 1] + lv.u[q - sy] + lv.u[q + sy] + lv.u[q - sz] + lv.u[q + sz];
                    lv.r[q] = lv.rhs[q] + s - 6.0 * lv.u[q];
                }
            }
        });
    }
    // coarse rhs = 0.5 * P^T r_fine (gather form)
    void restrict_to(const Level& f, Level& c) {
        pool->parallel_for(c.nz, [&](long K) {
            for (int J = 0; J < c.ny; ++J)
                for (int I = 0; I < c.nx; ++I) {
                    size_t qc = c.idx(I, J, (int)K);
                    if (c.fix[qc]) { c.rhs[qc] = 0.0; continue; }
                    double s = 0.0;
                    for (int dk = -1; dk <= 1; ++dk) {
                        int k = 2 * (int)K + dk;
                        if (k < 0 || k >= f.nz) continue;
                        double wk = dk == 0 ? 1.0 : 0.5;
                        for (int dj = -1; dj <= 1; ++dj) {
                            int j = 2 * J + dj;
                            if (j < 0 || j >= f.ny) continue;
                            double wj = dj == 0 ? 1.0 : 0.5;
                            for (int di = -1; di <= 1; ++di) {
                                int i = 2 * I + di;
                                if (i < 0 || i >= f.nx) continue;
                                double wi = di == 0 ? 1.0 : 0.5;
                                s += (wk * wj * wi) * f.r[f.idx(i, j, k)];
                            }
                        }
                    }
                    c.rhs[qc] = 0.5 * s;
                }
        });
    }
    // u_fine += P u_coarse at free fine nodes
    void prolong_add(const Level& c, Level& f) {
        pool->parallel_for(f.nz, [&](long k) {
            int k0 = (int)k / 2, k1 = ((int)k + 1) / 2;
            double wk1 = (k & 1) ? 0.5 : 0.0, wk0 = (k & 1) ? 0.5 : 1.0;
            for (int j = 0; j < f.ny; ++j) {
                int j0 = j / 2, j1 = (j + 1) / 2;
                double wj1 = (j & 1) ? 0.5 : 0.0, wj0 = (j & 1) ? 0.5 : 1.0;
                for (int i = 0; i < f.nx; ++i) {
                    size_t q = f.idx(i, j, (int)k);
                    if (f.fix[q]) continue;
                    int i0 = i / 2, i1 = (i + 1) / 2;
                    double wi1 = (i & 1) ? 0.5 : 0.0, wi0 = (i & 1) ? 0.5 : 1.0;
                    double s = 0.0;
                    s += wk0 * wj0 * wi0 * c.u[c.idx(i0, j0, k0)];
                    if (wi1 != 0.0) s += wk0 * wj0 * wi1 * c.u[c.idx(i1, j0, k0)];
                    if (wj1 != 0.0) {
                        s += wk0 * wj1 * wi0 * c.u[c.idx(i0, j1, k0)];
                        if (wi1 != 0.0) s += wk0 * wj1 * wi1 * c.u[c.idx(i1, j1, k0)];
                    }
                    if (wk1 != 0.0) {
                        s += wk1 * wj0 * wi0 * c.u[c.idx(i0, j0, k1)];
                        if (wi1 != 0.0) s += wk1 * wj0 * wi1 * c.u[c.idx(i1, j0, k1)];
                        if (wj1 != 0.0) {
                            s += wk1 * wj1 * wi0 * c.u[c.idx(i0, j1, k1)];
                            if (wi1 != 0.0) s += wk1 * wj1 * wi1 * c.u[c.idx(i1, j1, k1)];
                        }
                    }
                    f.u[q] += s;
                }
            }
        });
    }
    void zero(std::vector<double>& v) {
        size_t n = v.size(), chunk = 1 << 16;
        long nch = (long)((n + chunk - 1) / chunk);
        pool->parallel_for(nch, [&](long c) {
            size_t a = c * chunk, b = std::min(n, a + chunk);
            std::memset(v.data() + a, 0, (b - a) * sizeof(double));
        });
    }
    // symmetric V-cycle: solve S u = rhs on level l from u = 0
    void vcycle(int l) {
        Level& lv = L[l];
        zero(lv.u);
        if (l + 1 == (int)L.size()) {
            for (int s = 0; s < coarse_sweeps; ++s) { gs_color(lv, 0); gs_color(lv, 1); gs_color(lv, 1); gs_color(lv, 0); }
            return;
        }
        for (int s = 0; s < nu; ++s) { gs_color(lv, 0); gs_color(lv, 1); }
        residual(lv);
        restrict_to(lv, L[l + 1]);
        vcycle(l + 1);
        prolong_add(L[l + 1], lv);
        for (int s = 0; s < nu; ++s) { gs_color(lv, 1); gs_color(lv, 0); }
    }
    void build_hierarchy(int nx, int ny, int nz, const uint8_t* fix0) {
        L.clear();
        const std::vector<mqlv::Dims> D = mqlv::hierarchy(nx, ny, nz);
        for (size_t l = 0; l < D.size(); ++l) {
            Level lv;
            lv.nx = D[l].nx; lv.ny = D[l].ny; lv.nz = D[l].nz;
            lv.fix.assign(lv.n(), 0);
            if (l == 0) lv.fix.assign(fix0, fix0 + lv.n());
            else mqlv::coarse_fix(D[l - 1], L.back().fix.data(), D[l], lv.fix.data());
            lv.u.assign(lv.n(), 0.0); lv.rhs.assign(lv.n(), 0.0); lv.r.assign(lv.n(), 0.0);
            L.push_back(std::move(lv));
        }
    }
};

// Sum of f(q) over the grid in a fixed order: each row in i order, the rows of a plane in j order,
// the planes in k order (thread-count independent, and the order the device solver reproduces).
template <class F>
double ordered_sum(mq::Pool& pool, int nx, int ny, int nz, F f) {
    std::vector<double> part(nz, 0.0);
    pool.parallel_for(nz, [&](long k) {
        double plane = 0.0;
        for (int j = 0; j < ny; ++j) {
            const size_t base = (size_t)nx * ((size_t)j + (size_t)ny * k);
            double row = 0.0;
            for (int i = 0; i < nx; ++i) row += f(base + i);
            plane += row;
        }
        part[k] = plane;
    });
    double s = 0.0;
    for (int k = 0; k < nz; ++k) s += part[k];
    return s;
}

// per-plane maxima, combined in plane order
template <class F>
double plane_max(mq::Pool& pool, int nz, F f) {
    std::vector<double> part(nz, 0.0);
    pool.parallel_for(nz, [&](long k) { part[k] = f((int)k); });
    double s = 0.0;
    for (int k = 0; k < nz; ++k) s = std::max(s, part[k]);
    return s;
}

}  // namespace

extern "C" {

void mq_geom_default(mq_geom* g) {
    if (!g) return;
    std::memset(g, 0, sizeof(*g));
    g->de = 6.35; g->coef = 0.323; g->q1_start = 3.0; g->q1_len = 12.0; g->alpha = 0.02;
    g->gap = 1.0; g->plate = 1.6; g->hole_d = 7.0; g->q2_len = 3.0; g->stem_d = 4.6;
    g->q2_flare_bug = 1; g->grow = 0.0; g->tilt_mode = 0; g->ac_mode = 0;
    g->n_xy = 160; g->h_mm = 0.1;
}

mq_status mq_geom_dims(const mq_geom* g, int32_t dims[3]) {
    if (!g || !dims || g->n_xy < 3 || !(g->h_mm > 0)) return MQ_ERR_INVALID;
    dims[0] = g->n_xy; dims[1] = g->n_xy; dims[2] = geom_nz(g);
    return dims[2] >= 3 ? MQ_OK : MQ_ERR_INVALID;
}

double mq_geom_axis_mm(const mq_geom* g) { return g ? geom_axis(g) : 0.0; }

void mq_geom_layers(const mq_geom* g, double layers[8]) {
    if (!g || !layers) return;
    Layers L = layers_of(g);
    for (int i = 0; i < 8; ++i) layers[i] = L.l[i];
}

mq_status mq_geom_classify(const mq_geom* g, uint8_t* elec, size_t n) {
    int32_t d[3];
    if (mq_geom_dims(g, d) != MQ_OK || !elec) return MQ_ERR_INVALID;
    if (n != (size_t)d[0] * d[1] * d[2]) return MQ_ERR_INVALID;
    Layers L = layers_of(g);
    mq::Pool pool(0);
    pool.parallel_for(d[2], [&](long k) {
        for (int j = 0; j < d[1]; ++j)
            for (int i = 0; i < d[0]; ++i)
                elec[(size_t)i + (size_t)d[0] * ((size_t)j + (size_t)d[1] * k)] = classify(g, L, i, j, (int)k);
    });
    return MQ_OK;
}

mq_status mq_geom_basis_problem(const mq_geom* g, int32_t basis, uint8_t* mask, double* fixed,
                                size_t n, double* outer_bc) {
    if (basis < 0 || basis > 5 || !mask || !fixed) return MQ_ERR_INVALID;
    mq_status st = mq_geom_classify(g, mask, n);
    if (st != MQ_OK) return st;
    for (size_t q = 0; q < n; ++q) {
        uint8_t e = mask[q];
        fixed[q] = e ? basis_value(basis, e, g->ac_mode) : 0.0;
        mask[q] = e ? 1 : 0;
    }
    if (outer_bc) *outer_bc = basis == MQ_BASIS_DC_BOX ? 1.0 : 0.0;
    return MQ_OK;
}

mq_status mq_laplace_solve(int32_t nx, int32_t ny, int32_t nz, const uint8_t* mask,
                           const double* fixed, double outer_bc, double tol, int32_t threads,
                           double* phi, mq_solve_stats* stats) {
    if (nx < 3 || ny < 3 || nz < 3 || !mask || !fixed || !phi || !(tol > 0)) return MQ_ERR_INVALID;
    auto t0 = std::chrono::steady_clock::now();
    mq::Pool pool(threads);
    const size_t n = (size_t)nx * ny * nz;
    const size_t sy = nx, sz = (size_t)nx * ny;
    std::vector<uint8_t> fix(n);
    double maxfix = 0.0;
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                size_t q = (size_t)i + sy * j + sz * k;
                bool face = i == 0 || j == 0 || k == 0 || i == nx - 1 || j == ny - 1 || k == nz - 1;
                if (mask[q]) { fix[q] = 1; phi[q] = fixed[q]; maxfix = std::max(maxfix, std::fabs(fixed[q])); }
                else if (face) { fix[q] = 1; phi[q] = outer_bc; }
                else { fix[q] = 0; phi[q] = outer_bc; }
            }
    double scale = std::max(maxfix, std::fabs(outer_bc));
    if (!(scale > 0)) scale = 1.0;
    const double target = tol * scale;

    Solver S;
    S.pool = &pool;
    S.build_hierarchy(nx, ny, nz, fix.data());
    Level& l0 = S.L[0];
    std::vector<double> r(n, 0.0), p(n, 0.0), qv(n, 0.0);

    auto true_residual = [&]() {  // r = sum nb - 6 phi at free nodes; returns max |r|
        return plane_max(pool, nz, [&](int k) {
            double m = 0.0;
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    size_t q = (size_t)i + sy * j + sz * k;
                    if (fix[q]) { r[q] = 0.0; continue; }
                    double s = phi[q - 1] + phi[q + 1] + phi[q - sy] + phi[q + sy] + phi[q - sz] + phi[q + sz];
                    r[q] = s - 6.0 * phi[q];
                    m = std::max(m, std::fabs(r[q]));
                }
            return m;
        });
    };
    auto precond = [&]() {  // l0.u = M^-1 r
        std::memcpy(l0.rhs.data(), r.data(), n * sizeof(double));
        S.vcycle(0);
    };
    auto dot = [&](const std::vector<double>& a, const std::vector<double>& b) {
        return ordered_sum(pool, nx, ny, nz, [&](size_t q) { return a[q] * b[q]; });
    };

    double rmax = true_residual();
    int it = 0;
    const int max_it = 2000;
    bool converged = rmax <= target;
    while (!converged && it < max_it) {
        // (re)start PCG from the current iterate
        precond();
        std::memcpy(p.data(), l0.u.data(), n * sizeof(double));
        double rz = dot(r, l0.u);
        int inner = 0;
        while (it < max_it) {
            // q = S p (p vanishes at fixed nodes), and p . q
            double pq = ordered_sum(pool, nx, ny, nz, [&](size_t q) {
                if (fix[q]) { qv[q] = 0.0; return 0.0; }
                double nb = p[q - 1] + p[q + 1] + p[q - sy] + p[q + sy] + p[q - sz] + p[q + sz];
                qv[q] = 6.0 * p[q] - nb;
                return p[q] * qv[q];
            });
            if (!(pq > 0)) break;
            double alpha = rz / pq;
            rmax = plane_max(pool, nz, [&](int k) {
                double m = 0.0;
                size_t base = sz * k;
                for (size_t q = base; q < base + sz; ++q) {
                    phi[q] += alpha * p[q];
                    r[q] -= alpha * qv[q];
                    m = std::max(m, std::fabs(r[q]));
                }
                return m;
            });
            ++it; ++inner;
            if (rmax <= target || inner >= 200) break;
            precond();
            double rz_new = dot(r, l0.u);
            double beta = rz_new / rz;
            rz = rz_new;
            pool.parallel_for(nz, [&](long k) {
                size_t base = sz * k;
                for (size_t q = base; q < base + sz; ++q) p[q] = l0.u[q] + beta * p[q];
            });
        }
        rmax = true_residual();
        converged = rmax <= target;
        if (!converged && inner == 0) break;
    }
    if (stats) {
        stats->iterations = it;
        stats->converged = converged ? 1 : 0;
        stats->final_residual = rmax / scale;
        stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    return converged ? MQ_OK : MQ_ERR_NOT_CONVERGED;
}

mq_status mq_efield_central(const double* phi, int32_t nx, int32_t ny, int32_t nz, double h_m, float* e4) {
    if (!phi || !e4 || nx < 2 || ny < 2 || nz < 2 || !(h_m > 0)) return MQ_ERR_INVALID;
    mq::Pool pool(0);
    const size_t sy = nx, sz = (size_t)nx * ny;
    pool.parallel_for(nz, [&](long k) {
        int km = k > 0 ? (int)k - 1 : 0, kp = k + 1 < nz ? (int)k + 1 : nz - 1;
        for (int j = 0; j < ny; ++j) {
            int jm = j > 0 ? j - 1 : 0, jp = j + 1 < ny ? j + 1 : ny - 1;
            for (int i = 0; i < nx; ++i) {
                int im = i > 0 ? i - 1 : 0, ip = i + 1 < nx ? i + 1 : nx - 1;
                size_t q = (size_t)i + sy * j + sz * k;
                // d(a, b, da) = -(phi[b] - phi[a]) / da  (channel.rs:172)
                double ex = -(phi[(size_t)ip + sy * j + sz * k] - phi[(size_t)im + sy * j + sz * k]) / ((double)(ip - im) * h_m);
                double ey = -(phi[(size_t)i + sy * jp + sz * k] - phi[(size_t)i + sy * jm + sz * k]) / ((double)(jp - jm) * h_m);
                double ez = -(phi[(size_t)i + sy * j + sz * kp] - phi[(size_t)i + sy * j + sz * km]) / ((double)(kp - km) * h_m);
                e4[4 * q + 0] = (float)ex;
                e4[4 * q + 1] = (float)ey;
                e4[4 * q + 2] = (float)ez;
                e4[4 * q + 3] = 0.0f;
            }
        }
    });
    return MQ_OK;
}

mq_status mq_channel_basis(const mq_geom* g, int32_t basis, double tol, int32_t threads,
                           float* e4, double* phi_out, mq_solve_stats* stats) {
    return mq_channel_basis_ex(g, basis, tol, threads, -1, e4, phi_out, stats);
}

mq_status mq_channel_basis_ex(const mq_geom* g, int32_t basis, double tol, int32_t threads, int32_t device,
                              float* e4, double* phi_out, mq_solve_stats* stats) {
    int32_t d[3];
    if (mq_geom_dims(g, d) != MQ_OK || !e4 || basis < 0 || basis > 5) return MQ_ERR_INVALID;
    size_t n = (size_t)d[0] * d[1] * d[2];
    std::vector<uint8_t> mask(n);
    std::vector<double> fixed(n);
    double outer = 0.0;
    mq_status st = mq_geom_basis_problem(g, basis, mask.data(), fixed.data(), n, &outer);
    if (st != MQ_OK) return st;
    std::unique_ptr<double[]> own;
    double* phi = phi_out;
    if (!phi) { own.reset(new (std::nothrow) double[n]); phi = own.get(); if (!phi) return MQ_ERR_NOMEM; }
    st = device >= 0 ? mq_laplace_solve_device(d[0], d[1], d[2], mask.data(), fixed.data(), outer, tol, device, phi, stats)
                     : mq_laplace_solve(d[0], d[1], d[2], mask.data(), fixed.data(), outer, tol, threads, phi, stats);
    if (st != MQ_OK) return st;
    st = mq_efield_central(phi, d[0], d[1], d[2], g->h_mm * 1e-3, e4);
    if (st != MQ_OK) return st;
    if (basis == MQ_BASIS_RF)
        for (size_t q = 0; q < n; ++q) e4[4 * q + 3] = (float)mask[q];  // RF.w = conductor mask (channel.rs:213)
    return MQ_OK;
}

mq_status mq_dc_combine(size_t n, const float* const dc4[4], const double v[4], float* out4) {
    if (!dc4 || !v || !out4) return MQ_ERR_INVALID;
    float vf[4];
    for (int b = 0; b < 4; ++b) vf[b] = (float)v[b];
    mq::Pool pool(0);
    const size_t chunk = 1 << 16;
    long nch = (long)((n + chunk - 1) / chunk);
    pool.parallel_for(nch, [&](long c) {
        size_t a = c * chunk, e = std::min(n, a + chunk);
        for (size_t q = a; q < e; ++q) {
            float acc[3] = {0.0f, 0.0f, 0.0f};
            for (int b = 0; b < 4; ++b) {
                if (!dc4[b]) continue;
                for (int d = 0; d < 3; ++d) acc[d] += vf[b] * dc4[b][4 * q + d];
            }
            out4[4 * q + 0] = acc[0]; out4[4 * q + 1] = acc[1]; out4[4 * q + 2] = acc[2]; out4[4 * q + 3] = 0.0f;
        }
    });
    return MQ_OK;
}

}  // extern "C"
