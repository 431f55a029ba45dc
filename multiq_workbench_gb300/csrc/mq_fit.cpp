// Resonance-curve fits and the secular-frequency terrain: the callers that turn the per-frequency
// outcome counts of a batch sweep into R = f0 / FWHM.  Host code, compiled without FMA contraction;
// every expression keeps the reference's operand order so a fit of the same counts gives the same
// parameters (simulation/mqviz/src/fit.rs, terrain.rs, analysis.rs:10-18, stats.rs:152-171).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "mq_fit.h"
#include "mq_grid.h"

namespace {

constexpr double kLn2 = 0.693147180559945309417232121458176568;
constexpr double kTau = 6.28318530717958647692528676655900577;
constexpr double kAmu = 1.6605390666e-27;   // world.rs:13
constexpr double kQe = 1.602176634e-19;     // world.rs:14

inline double clampd(double x, double lo, double hi) {   // f64::clamp: NaN stays NaN
    if (x < lo) x = lo;
    if (x > hi) x = hi;
    return x;
}

// ------------------------------------------------------------------ statistics generator (stats.rs:152-171)

struct Rng {
    uint64_t s;
    double u() {
        s ^= s << 13;
        s ^= s >> 7;
        s ^= s << 17;
        return (double)(s >> 11) / 9007199254740992.0;
    }
    double normal() {
        const double a = std::fmax(u(), 1e-300);
        const double b = u();
        return std::sqrt(-2.0 * std::log(a)) * std::cos(kTau * b);
    }
    uint64_t binomial(uint64_t n, double p) {
        const double nf = (double)n;
        if (n > 400 && p * (1.0 - p) * nf > 50.0) {
            const double x = nf * p + std::sqrt(nf * p * (1.0 - p)) * normal();
            return (uint64_t)clampd(std::round(x), 0.0, nf);
        }
        uint64_t k = 0;
        for (uint64_t i = 0; i < n; ++i) k += u() < p;
        return k;
    }
};

// ------------------------------------------------------------------ shapes (fit.rs:9-33)

typedef double P4[4];

double shape_g(int sh, double d, double w) {
    if (sh == MQ_SHAPE_LORENTZ) {
        const double u = 2.0 * d / w;
        return 1.0 / (1.0 + u * u);
    }
    return std::exp(-4.0 * kLn2 * d * d / (w * w));
}

// d g / d d and d g / d w
void shape_dg(int sh, double d, double w, double* gd, double* gw) {
    if (sh == MQ_SHAPE_LORENTZ) {
        const double u = 2.0 * d / w;
        const double g = 1.0 / (1.0 + u * u);
        const double g2 = g * g;
        *gd = -g2 * 2.0 * u * 2.0 / w;
        *gw = g2 * 2.0 * u * u / w;
        return;
    }
    const double g = shape_g(sh, d, w);
    *gd = g * (-8.0 * kLn2 * d / (w * w));
    *gw = g * 8.0 * kLn2 * d * d / (w * w * w);
}

inline double model(int sh, const double* p, double x) { return p[0] + p[1] * shape_g(sh, x - p[2], p[3]); }

// Gauss-Jordan with partial pivoting; the pivot is the last row of largest magnitude (Iterator::max_by).
bool solve4(const double a[4][4], const double b[4], double out[4]) {
    double m[4][5];
    for (int i = 0; i < 4; ++i) {
        for (int j = 0; j < 4; ++j) m[i][j] = a[i][j];
        m[i][4] = b[i];
    }
    for (int c = 0; c < 4; ++c) {
        int piv = c;
        for (int i = c + 1; i < 4; ++i)
            if (std::fabs(m[i][c]) >= std::fabs(m[piv][c])) piv = i;
        if (!(std::fabs(m[piv][c]) >= 1e-300)) return false;   // also refuses NaN pivots
        if (piv != c)
            for (int k = 0; k < 5; ++k) std::swap(m[c][k], m[piv][k]);
        for (int r = 0; r < 4; ++r) {
            if (r == c) continue;
            const double f = m[r][c] / m[c][c];
            for (int k = c; k < 5; ++k) m[r][k] -= f * m[c][k];
        }
    }
    for (int i = 0; i < 4; ++i) out[i] = m[i][4] / m[i][i];
    return true;
}

bool invert4(const double a[4][4], double out[4][4]) {
    for (int c = 0; c < 4; ++c) {
        double e[4] = {0, 0, 0, 0}, s[4];
        e[c] = 1.0;
        if (!solve4(a, e, s)) return false;
        for (int r = 0; r < 4; ++r) out[r][c] = s[r];
    }
    return true;
}

double chi2_of(int sh, const double* p, const std::vector<double>& xs, const std::vector<double>& ys,
               const std::vector<double>& sg) {
    double s = 0.0;
    for (size_t i = 0; i < xs.size(); ++i) {
        const double r = (ys[i] - model(sh, p, xs[i])) / sg[i];
        s += r * r;
    }
    return s;
}

struct Bounds { double x_lo, x_hi, w_lo, w_hi; };

inline void clamp_p(double* p, const Bounds& b) {
    p[2] = clampd(p[2], b.x_lo, b.x_hi);
    p[3] = clampd(p[3], b.w_lo, b.w_hi);
}

// Jacobian row of the weighted residual at point i
inline void jac_row(int sh, const double* p, double x, double s, double j[4]) {
    const double d = x - p[2];
    double gd, gw;
    shape_dg(sh, d, p[3], &gd, &gw);
    const double g = shape_g(sh, d, p[3]);
    j[0] = 1.0 / s;
    j[1] = g / s;
    j[2] = -p[1] * gd / s;
    j[3] = p[1] * gw / s;
}

struct LmResult { P4 p; double chi2; bool conv; };

// Levenberg-Marquardt from a start (fit.rs:93-129)
LmResult lm(int sh, const double* start, const std::vector<double>& xs, const std::vector<double>& ys,
            const std::vector<double>& sg, const Bounds& b) {
    LmResult R;
    std::memcpy(R.p, start, sizeof(P4));
    clamp_p(R.p, b);
    double chi = chi2_of(sh, R.p, xs, ys, sg);
    double lam = 1e-3;
    bool conv = false;
    for (int it = 0; it < 200; ++it) {
        double jtj[4][4] = {{0}}, jtr[4] = {0, 0, 0, 0};
        for (size_t i = 0; i < xs.size(); ++i) {
            double j[4];
            jac_row(sh, R.p, xs[i], sg[i], j);
            const double r = (ys[i] - model(sh, R.p, xs[i])) / sg[i];
            for (int a = 0; a < 4; ++a) {
                jtr[a] += j[a] * r;
                for (int c = 0; c < 4; ++c) jtj[a][c] += j[a] * j[c];
            }
        }
        bool improved = false;
        for (int t = 0; t < 12; ++t) {
            double a[4][4];
            std::memcpy(a, jtj, sizeof(a));
            for (int k = 0; k < 4; ++k) a[k][k] += lam * std::fmax(jtj[k][k], 1e-12);
            double dp[4];
            if (!solve4(a, jtr, dp)) {
                lam *= 10.0;
                continue;
            }
            double q[4] = {R.p[0] + dp[0], R.p[1] + dp[1], R.p[2] + dp[2], R.p[3] + dp[3]};
            clamp_p(q, b);
            const double c2 = chi2_of(sh, q, xs, ys, sg);
            if (std::isfinite(c2) && c2 < chi) {
                const double rel = (chi - c2) / std::fmax(chi, 1e-300);
                std::memcpy(R.p, q, sizeof(P4));
                chi = c2;
                lam = std::fmax(lam * 0.3, 1e-9);
                improved = true;
                if (rel < 1e-10) conv = true;
                break;
            }
            lam *= 5.0;
        }
        if (!improved) conv = true;
        if (conv) break;
    }
    R.chi2 = chi;
    R.conv = conv;
    return R;
}

double half_max_width(const std::vector<double>& xs, const std::vector<double>& ys, double base, size_t imax) {
    const double half = base + 0.5 * (ys[imax] - base);
    double lo = xs[0], hi = xs[xs.size() - 1];
    for (size_t i = imax; i >= 1; --i)
        if (ys[i - 1] < half) {
            lo = xs[i - 1] + (half - ys[i - 1]) / (ys[i] - ys[i - 1]) * (xs[i] - xs[i - 1]);
            break;
        }
    for (size_t i = imax; i + 1 < xs.size(); ++i)
        if (ys[i + 1] < half) {
            hi = xs[i] + (ys[i] - half) / (ys[i] - ys[i + 1]) * (xs[i + 1] - xs[i]);
            break;
        }
    return std::fmax(hi - lo, 1e-6);
}

Bounds bounds_of(const std::vector<double>& xs) {
    const double lo = xs[0], hi = xs[xs.size() - 1];
    const double dx = (hi - lo) / (double)(xs.size() - 1);
    return Bounds{lo - 0.2 * (hi - lo), hi + 0.2 * (hi - lo), 0.3 * dx, 3.0 * (hi - lo)};
}

// Best of three starting widths (and an optional given start) (fit.rs:153-170)
LmResult fit_shape(int sh, const std::vector<double>& xs, const std::vector<double>& ys, const std::vector<double>& sg,
                   const double* init) {
    const Bounds b = bounds_of(xs);
    const size_t n = xs.size();
    std::vector<double> sm(n);
    for (size_t i = 0; i < n; ++i) {
        const size_t a = i ? i - 1 : 0, c = i + 1 < n ? i + 1 : n - 1;
        sm[i] = (ys[a] + ys[i] + ys[c]) / 3.0;
    }
    size_t imax = 0;   // the last index of the largest smoothed value (Iterator::max_by)
    for (size_t i = 1; i < n; ++i)
        if (sm[i] >= sm[imax]) imax = i;
    double base = INFINITY;
    for (double y : ys) base = std::fmin(base, y);
    base = std::fmax(base, 0.0);
    if (!std::isfinite(base)) base = 0.0;
    const double amp = std::fmax(ys[imax] - base, 1e-9);
    const double w0 = half_max_width(xs, ys, base, imax);
    std::vector<std::vector<double>> starts;
    if (init) starts.push_back(std::vector<double>(init, init + 4));
    for (double f : {1.0, 0.5, 2.0}) starts.push_back({base, amp, xs[imax], clampd(w0 * f, b.w_lo, b.w_hi)});
    LmResult best{};
    bool have = false;
    for (const auto& s : starts) {
        LmResult r = lm(sh, s.data(), xs, ys, sg, b);
        if (!have || r.chi2 < best.chi2) {
            best = r;
            have = true;
        }
    }
    return best;
}

bool covariance(int sh, const double* p, const std::vector<double>& xs, const std::vector<double>& sg,
                double cov[4][4]) {
    double jtj[4][4] = {{0}};
    for (size_t i = 0; i < xs.size(); ++i) {
        double j[4];
        jac_row(sh, p, xs[i], sg[i], j);
        for (int a = 0; a < 4; ++a)
            for (int c = 0; c < 4; ++c) jtj[a][c] += j[a] * j[c];
    }
    return invert4(jtj, cov);
}

// covariance, scaled errors and R (fit.rs:193-202)
bool finish(int sh, const double* p, double chi2, bool conv, const std::vector<double>& xs,
            const std::vector<double>& sg, mq_res_fit* out) {
    double cov[4][4];
    if (!covariance(sh, p, xs, sg, cov)) return false;
    std::memset(out, 0, sizeof(*out));
    const int64_t dof = (int64_t)xs.size() - 4;
    const double scale = (dof > 0 && chi2 / (double)dof > 1.0) ? std::sqrt(chi2 / (double)dof) : 1.0;
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) cov[r][c] *= scale * scale;
    out->shape = sh;
    out->converged = conv ? 1 : 0;
    for (int k = 0; k < 4; ++k) {
        out->p[k] = p[k];
        out->e[k] = std::sqrt(std::fmax(cov[k][k], 0.0));
        for (int c = 0; c < 4; ++c) out->cov[4 * k + c] = cov[k][c];
    }
    out->chi2 = chi2;
    out->chi2_flat = NAN;
    out->dof = dof;
    out->scale = scale;
    out->n_pts = xs.size();
    const double f0 = p[2], w = p[3];
    out->r = f0 / w;
    const double gf = 1.0 / w, gw = -f0 / (w * w);
    const double v = gf * gf * cov[2][2] + gw * gw * cov[3][3] + 2.0 * gf * gw * cov[2][3];
    out->r_err = std::sqrt(std::fmax(v, 0.0));
    out->r_boot_mean = out->r_boot_sd = out->f0_boot_sd = NAN;
    return true;
}

// Jeffreys floor keeps sigma finite where the model predicts ~0 or ~1 (fit.rs:204-209)
inline double bin_var(double p, uint64_t n) {
    const double ni = (double)n;
    double pj = clampd(p, 0.0, 1.0);
    pj = std::fmax(pj, 0.5 / (ni + 1.0));
    pj = std::fmin(pj, 1.0 - 0.5 / (ni + 1.0));
    return pj * (1.0 - pj) / ni;
}

int32_t binomial_shape(int sh, const double* xs_in, const uint64_t* ks_in, const uint64_t* ns_in, size_t m,
                       uint64_t boot, uint64_t seed, mq_res_fit* out) {
    std::vector<double> x, y;
    std::vector<uint64_t> k, n;
    for (size_t i = 0; i < m; ++i)
        if (ns_in[i] > 0) {
            x.push_back(xs_in[i]);
            k.push_back(ks_in[i]);
            n.push_back(ns_in[i]);
        }
    if (x.size() < 6) return MQ_ERR_INVALID;
    const size_t L = x.size();
    for (size_t i = 0; i < L; ++i) y.push_back((double)k[i] / (double)n[i]);
    std::vector<double> sg(L);
    for (size_t i = 0; i < L; ++i) sg[i] = std::sqrt(bin_var(((double)k[i] + 0.5) / ((double)n[i] + 1.0), n[i]));
    LmResult f = fit_shape(sh, x, y, sg, nullptr);
    for (int it = 0; it < 3; ++it) {
        for (size_t i = 0; i < L; ++i) sg[i] = std::sqrt(bin_var(model(sh, f.p, x[i]), n[i]));
        f = fit_shape(sh, x, y, sg, f.p);
    }
    for (size_t i = 0; i < L; ++i) sg[i] = std::sqrt(bin_var(model(sh, f.p, x[i]), n[i]));
    const double chi2 = chi2_of(sh, f.p, x, y, sg);
    if (!finish(sh, f.p, chi2, f.conv, x, sg, out)) return 1;
    {
        uint64_t ks = 0, nn = 0;
        for (size_t i = 0; i < L; ++i) {
            ks += k[i];
            nn += n[i];
        }
        const double pbar = (double)ks / (double)nn;
        double c = 0.0;
        for (size_t i = 0; i < L; ++i) {
            const double d = y[i] - pbar;
            c += d * d / bin_var(pbar, n[i]);
        }
        out->chi2_flat = c;
    }
    if (boot > 0) {
        Rng rng{mq_rng_seed(seed ^ 0xB007ull)};
        std::vector<double> rs, fs, yb(L), sb(L);
        const Bounds bnds = bounds_of(x);
        for (uint64_t r = 0; r < boot; ++r) {
            for (size_t i = 0; i < L; ++i)
                yb[i] = (double)rng.binomial(n[i], clampd(model(sh, out->p, x[i]), 0.0, 1.0)) / (double)n[i];
            for (size_t i = 0; i < L; ++i) sb[i] = std::sqrt(bin_var(model(sh, out->p, x[i]), n[i]));
            const LmResult pb = lm(sh, out->p, x, yb, sb, bnds);
            rs.push_back(pb.p[2] / pb.p[3]);
            fs.push_back(pb.p[2]);
        }
        auto sd = [](const std::vector<double>& v, double* mean) {
            double s = 0.0;
            for (double a : v) s += a;
            const double m = s / (double)v.size();
            double q = 0.0;
            for (double a : v) q += (a - m) * (a - m);
            *mean = m;
            return std::sqrt(q / ((double)v.size() - 1.0));
        };
        double mr, mf;
        out->r_boot_sd = sd(rs, &mr);
        out->r_boot_mean = mr;
        out->f0_boot_sd = sd(fs, &mf);
        out->has_boot = 1;
    }
    return MQ_OK;
}

bool shape_ok(int32_t sh) { return sh == MQ_SHAPE_LORENTZ || sh == MQ_SHAPE_GAUSS; }

// ------------------------------------------------------------------ terrain (terrain.rs, world.rs:187-231)

// trilinear value of a float4 node field, the clamped-cell form of world.rs:191-201
void trif(int nx, int ny, int nz, double h, const float* v4, const double x[3], double e[3]) {
    const double g[3] = {x[0] / h, x[1] / h, x[2] / h};
    auto cell = [](double gg, int n) {
        const double c = gg > 0.0 ? std::floor(gg) : 0.0;   // (g.max(0.0) as usize), NaN -> 0
        return c >= (double)(n - 2) ? (size_t)(n - 2) : (size_t)c;
    };
    const size_t i = cell(g[0], nx), j = cell(g[1], ny), k = cell(g[2], nz);
    const double tx = g[0] - (double)i, ty = g[1] - (double)j, tz = g[2] - (double)k;
    e[0] = e[1] = e[2] = 0.0;
    for (int di = 0; di < 2; ++di)
        for (int dj = 0; dj < 2; ++dj)
            for (int dk = 0; dk < 2; ++dk) {
                const double wx = di ? tx : 1.0 - tx, wy = dj ? ty : 1.0 - ty, wz = dk ? tz : 1.0 - tz;
                const size_t q = (i + di) + (size_t)nx * ((j + dj) + (size_t)ny * (k + dk));
                for (int d = 0; d < 3; ++d) e[d] += wx * wy * wz * (double)v4[4 * q + d];
            }
}

}  // namespace

extern "C" {

double mq_fit_model(int32_t shape, const double p[4], double x) { return model(shape, p, x); }

int32_t mq_fit_shape_sigma(int32_t shape, const double* xs, const double* ys, const double* sg, size_t n,
                           mq_res_fit* out) {
    if (!shape_ok(shape) || !xs || !ys || !sg || !out || n < 6) return MQ_ERR_INVALID;
    std::vector<double> x(xs, xs + n), y(ys, ys + n), s(sg, sg + n);
    const LmResult f = fit_shape(shape, x, y, s, nullptr);
    return finish(shape, f.p, f.chi2, f.conv, x, s, out) ? MQ_OK : 1;
}

int32_t mq_fit_binomial_shape(int32_t shape, const double* xs, const uint64_t* ks, const uint64_t* ns, size_t n,
                              uint64_t boot, uint64_t seed, mq_res_fit* out) {
    if (!shape_ok(shape) || !xs || !ks || !ns || !out) return MQ_ERR_INVALID;
    return binomial_shape(shape, xs, ks, ns, n, boot, seed, out);
}

int32_t mq_fit_binomial_curve(const double* xs, const uint64_t* ks, const uint64_t* ns, size_t n, uint64_t boot,
                              uint64_t seed, mq_res_fit* out) {
    if (!xs || !ks || !ns || !out) return MQ_ERR_INVALID;
    mq_res_fit best, cur;
    bool have = false;
    int32_t last = 1;
    for (int sh : {MQ_SHAPE_LORENTZ, MQ_SHAPE_GAUSS}) {
        last = binomial_shape(sh, xs, ks, ns, n, boot, seed, &cur);
        if (last == MQ_OK && (!have || cur.chi2 < best.chi2)) {
            best = cur;
            have = true;
        }
    }
    if (!have) return last == MQ_ERR_INVALID ? MQ_ERR_INVALID : 1;
    *out = best;
    return MQ_OK;
}

int32_t mq_fit_is_significant(const mq_res_fit* f, const double* xs, size_t n) {
    if (!f || !xs || n == 0) return 0;
    double lo = INFINITY, hi = -INFINITY;
    for (size_t i = 0; i < n; ++i) {
        lo = std::fmin(lo, xs[i]);
        hi = std::fmax(hi, xs[i]);
    }
    const double step = (hi - lo) / (double)((n > 2 ? n : 2) - 1);
    for (int k = 0; k < 4; ++k)
        if (!std::isfinite(f->e[k])) return 0;
    const double dchi = f->chi2_flat - f->chi2;
    return dchi >= MQ_FIT_MIN_DELTA_CHI2 && f->p[2] >= lo && f->p[2] <= hi && f->e[2] < 0.5 * (hi - lo) &&
           f->p[3] >= 0.5 * step && f->p[3] <= hi - lo && std::isfinite(f->r_err);
}

void mq_fit_r_mz(double mz, double dfdmz, double fwhm, double fwhm_err, double out[4]) {
    const double slope = std::fmax(std::fabs(dfdmz), 1e-12);
    const double d = fwhm / slope, de = fwhm_err / slope;
    out[0] = d;
    out[1] = de;
    out[2] = mz / d;
    out[3] = mz / (d * d) * de;
}

uint64_t mq_rng_seed(uint64_t seed) { return (seed * 0x9E3779B97F4A7C15ull) | 1ull; }

double mq_rng_uniform(uint64_t* state) {
    Rng r{*state};
    const double u = r.u();
    *state = r.s;
    return u;
}

void mq_rng_binomial_fill(uint64_t* state, const uint64_t* n, const double* p, size_t m, uint64_t* out) {
    Rng r{*state};
    for (size_t i = 0; i < m; ++i) out[i] = r.binomial(n[i], p[i]);
    *state = r.s;
}

double mq_mathieu_beta(double a, double q) {
    double b = std::sqrt(std::fmax(a + q * q / 2.0, 1e-12));
    auto cf = [&](double bb, double sgn) {
        double s = 0.0;
        for (int k = 11; k >= 1; --k) {
            const double kk = bb + sgn * 2.0 * (double)k;
            s = q * q / (kk * kk - a - s);
        }
        return s;
    };
    for (int it = 0; it < 60; ++it) {
        const double nb = std::sqrt(std::fmax(a + cf(b, 1.0) + cf(b, -1.0), 1e-12));
        if (std::fabs(nb - b) < 1e-12) {
            b = nb;
            break;
        }
        b = 0.5 * (b + nb);
    }
    return b;
}

double mq_sec_freq_khz(double g_rf, double g_dc, double qm, double v_rf, double f_rf) {
    const double om = kTau * f_rf;
    const double q = 2.0 * qm * std::fabs(g_rf) * v_rf / (om * om);
    const double a = -4.0 * qm * g_dc / (om * om);
    if (a + q * q / 2.0 <= 0.0 || q > 0.95) return NAN;
    return mq_mathieu_beta(a, q) * f_rf / 1e3 / 2.0;
}

int32_t mq_terrain_tables(int32_t nx, int32_t ny, int32_t nz, double h, double axis_m, const float* rf4,
                          const float* const dc4[4], size_t cap, double* z_mm, double* rf2, double* dc2, size_t* n_out) {
    if (nx < 2 || ny < 2 || nz < 3 || !(h > 0.0) || !rf4 || !dc4 || !z_mm || !rf2 || !dc2 || !n_out)
        return MQ_ERR_INVALID;
    for (int b = 0; b < 4; ++b)
        if (!dc4[b]) return MQ_ERR_INVALID;
    const double hh = 0.2e-3;
    auto jac = [&](const float* v, double z, double jm[2][2]) {
        for (int dj = 0; dj < 2; ++dj) {
            double p[3] = {axis_m, axis_m, z}, m[3] = {axis_m, axis_m, z};
            p[dj] += hh;
            m[dj] -= hh;
            double ep[3], em[3];
            trif(nx, ny, nz, h, v, p, ep);
            trif(nx, ny, nz, h, v, m, em);
            for (int di = 0; di < 2; ++di) jm[di][dj] = (ep[di] - em[di]) / (2.0 * hh);
        }
    };
    auto proj = [](const double j[2][2], double ux, double uy) {
        return ux * (j[0][0] * ux + j[0][1] * uy) + uy * (j[1][0] * ux + j[1][1] * uy);
    };
    size_t k = 0;
    double z = 0.3e-3;
    while (z < (double)(nz - 2) * h && z < 20.0e-3) {
        if (k >= cap) return MQ_ERR_INVALID;
        double jr[2][2];
        jac(rf4, z, jr);
        const double s11 = jr[0][0], s12 = 0.5 * (jr[0][1] + jr[1][0]), s22 = jr[1][1];
        const double th = 0.5 * std::atan2(2.0 * s12, s11 - s22);
        const double c = std::cos(th), sn = std::sin(th);
        z_mm[k] = z * 1e3;
        rf2[2 * k] = proj(jr, c, sn);
        rf2[2 * k + 1] = proj(jr, -sn, c);
        for (int b = 0; b < 4; ++b) {
            double jd[2][2];
            jac(dc4[b], z, jd);
            dc2[(b * cap + k) * 2] = proj(jd, c, sn);
            dc2[(b * cap + k) * 2 + 1] = proj(jd, -sn, c);
        }
        ++k;
        z += 0.1e-3;
    }
    *n_out = k;
    return MQ_OK;
}

int32_t mq_terrain_compute(size_t n, size_t cap, const double* rf2, const double* dc2, const double* mass,
                           const double* charge, size_t nsp, double v_rf, const double dc[4], double f_rf,
                           double* fx, double* fy) {
    if (n > cap || !rf2 || !dc2 || !mass || !charge || !dc || !fx || !fy) return MQ_ERR_INVALID;
    for (size_t s = 0; s < nsp; ++s) {
        const double qm = charge[s] * kQe / (mass[s] * kAmu);
        for (size_t k = 0; k < n; ++k) {
            double gdx = 0.0, gdy = 0.0;
            for (int b = 0; b < 4; ++b) {
                gdx += dc[b] * dc2[(b * cap + k) * 2];
                gdy += dc[b] * dc2[(b * cap + k) * 2 + 1];
            }
            fx[s * n + k] = mq_sec_freq_khz(rf2[2 * k], gdx, qm, v_rf, f_rf);
            fy[s * n + k] = mq_sec_freq_khz(rf2[2 * k + 1], gdy, qm, v_rf, f_rf);
        }
    }
    return MQ_OK;
}

double mq_terrain_dfdmz(size_t n, size_t cap, const double* z_mm, const double* rf2, const double* dc2, double mass,
                        double charge, double v_rf, const double dc[4], double f_rf) {
    if (n == 0 || n > cap || !z_mm) return NAN;
    const double eps = 0.01;
    const double m2[2] = {mass * (1.0 + eps), mass * (1.0 - eps)}, z2[2] = {charge, charge};
    std::vector<double> fx(2 * n), fy(2 * n);
    if (mq_terrain_compute(n, cap, rf2, dc2, m2, z2, 2, v_rf, dc, f_rf, fx.data(), fy.data()) != MQ_OK) return NAN;
    size_t k = 0;
    for (size_t i = 0; i < n; ++i)
        if (z_mm[i] >= 6.0) {
            k = i;
            break;
        }
    return (fx[k] - fx[n + k]) / (2.0 * eps * (mass / charge));
}

int32_t mq_secular_freq(const float* rf4, int32_t nx, int32_t ny, int32_t nz, double h, double axis_m, double qm,
                        double v_rf, double f_rf, double z_m, double* out) {
    if (!rf4 || !out || nx < 2 || ny < 2 || nz < 2 || !(h > 0.0) || !(f_rf > 0.0)) return MQ_ERR_INVALID;
    auto tri = [&](const double x[3], double e[3]) {
        const double g[3] = {x[0] / h, x[1] / h, x[2] / h};
        auto cell = [](double gg, int n) {
            const double c = gg > 0.0 ? std::floor(gg) : 0.0;
            return c >= (double)(n - 2) ? (size_t)(n - 2) : (size_t)c;
        };
        const size_t i = cell(g[0], nx), j = cell(g[1], ny), k = cell(g[2], nz);
        const double tx = g[0] - (double)i, ty = g[1] - (double)j, tz = g[2] - (double)k;
        e[0] = e[1] = e[2] = 0.0;
        for (int di = 0; di < 2; ++di)
            for (int dj = 0; dj < 2; ++dj)
                for (int dk = 0; dk < 2; ++dk) {
                    const double wx = di ? tx : 1.0 - tx, wy = dj ? ty : 1.0 - ty, wz = dk ? tz : 1.0 - tz;
                    const size_t q = (i + di) + (size_t)nx * ((j + dj) + (size_t)ny * (k + dk));
                    for (int d = 0; d < 3; ++d) e[d] += wx * wy * wz * (double)rf4[4 * q + d];
                }
    };
    const double a = axis_m, amp = 0.2e-3, w = kTau * f_rf;
    double x[3] = {a + amp / std::sqrt(2.0), a - amp / std::sqrt(2.0), z_m};
    double v[3] = {0.0, 0.0, 0.0};
    const double dt = 1.0 / f_rf / 200.0;
    const size_t n = (size_t)(4e-3 / dt);
    std::vector<double> cross;
    double prev = (x[0] - a) - (x[1] - a);
    double t = 0.0;
    *out = NAN;
    for (size_t s = 0; s < n; ++s) {
        double e[3];
        tri(x, e);
        const double sn = v_rf * std::sin(w * t);
        for (int d = 0; d < 2; ++d) v[d] += qm * sn * e[d] * dt;   // transverse only: z frozen at the slice
        for (int d = 0; d < 2; ++d) x[d] += v[d] * dt;
        t += dt;
        const double u = (x[0] - a) - (x[1] - a);
        if (prev < 0.0 && u >= 0.0) cross.push_back(t);
        prev = u;
        if (std::fabs(x[0] - a) > 2.5e-3 || std::fabs(x[1] - a) > 2.5e-3) return MQ_OK;
    }
    if (cross.size() < 3) return MQ_OK;
    *out = (double)(cross.size() - 1) / (cross.back() - cross.front());
    return MQ_OK;
}

}  // extern "C"
