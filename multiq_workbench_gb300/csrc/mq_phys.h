// Physics of the ion-trajectory path shared by host code (injection, constants) and the
// FP64 CUDA kernel.  Everything here is evaluated with IEEE double operations in a fixed
// order and without FMA contraction (host: -ffp-contract=off, device: --fmad=false), so
// the host, the FP64 kernel and any other conforming evaluator agree bit for bit.
//
// Reference (filiprumenovski/multiq-workbench):
//   integrator  simulation/mqviz/src/world.rs:265-314,385-422,437-536
//   switches    simulation/chsim/src/channel.rs:254-273,342-426; channel.metal:56-62,100-121
#pragma once
#include <stdint.h>
#include <math.h>

#if defined(__CUDACC__)
#define MQ_HD __host__ __device__ __forceinline__
#else
#define MQ_HD inline
#endif

namespace mqp {

constexpr double AMU = 1.6605390666e-27;   // channel.rs:11
constexpr double QE = 1.602176634e-19;     // channel.rs:12
constexpr double KB = 1.380649e-23;        // channel.rs:13

// ---------------------------------------------------------------- deterministic transcendentals
// sin/cos: exact reduction in turns, Taylor polynomials on [-pi/4, pi/4] (coefficients
// (-1)^k/(2k+1)! and (-1)^k/(2k)!, correctly rounded).  log: x = m 2^e with
// m in [sqrt(1/2), sqrt(2)), log m = 2 atanh((m-1)/(m+1)) summed as its odd power series.
MQ_HD double sin_poly(double x) {
    double z = x * x;
    double p = -0x1.ae7f3e733b81fp-41 + z * 0x1.952c77030ad4ap-49;
    p = 0x1.6124613a86d09p-33 + z * p;
    p = -0x1.ae64567f544e4p-26 + z * p;
    p = 0x1.71de3a556c734p-19 + z * p;
    p = -0x1.a01a01a01a01ap-13 + z * p;
    p = 0x1.1111111111111p-7 + z * p;
    p = -0x1.5555555555555p-3 + z * p;
    return x + (x * z) * p;
}
MQ_HD double cos_poly(double x) {
    double z = x * x;
    double p = 0x1.ae7f3e733b81fp-45 + z * -0x1.6827863b97d97p-53;
    p = -0x1.93974a8c07c9dp-37 + z * p;
    p = 0x1.1eed8eff8d898p-29 + z * p;
    p = -0x1.27e4fb7789f5cp-22 + z * p;
    p = 0x1.a01a01a01a01ap-16 + z * p;
    p = -0x1.6c16c16c16c17p-10 + z * p;
    p = 0x1.5555555555555p-5 + z * p;
    return (1.0 - 0.5 * z) + (z * z) * p;
}
// sin(2 pi u), cos(2 pi u)
MQ_HD void sincos2pi(double u, double* s, double* c) {
    u = u - floor(u);
    double t = 4.0 * u;
    double q = rint(t);
    double x = (t - q) * 0x1.921fb54442d18p+0;
    double sk = sin_poly(x), ck = cos_poly(x);
    int qi = ((int)q) & 3;
    if (qi == 0) { *s = sk; *c = ck; }
    else if (qi == 1) { *s = ck; *c = -sk; }
    else if (qi == 2) { *s = -sk; *c = -ck; }
    else { *s = -ck; *c = sk; }
}
MQ_HD double log_(double x) {
    int e;
    double m = frexp(x, &e);
    if (m < 0x1.6a09e667f3bcdp-1) { m = m * 2.0; e -= 1; }
    double f = m - 1.0;
    double s = f / (2.0 + f);
    double z = s * s;
    double r = 0x1.8618618618618p-5 + z * 0x1.642c8590b2164p-5;
    r = 0x1.af286bca1af28p-5 + z * r;
    r = 0x1.e1e1e1e1e1e1ep-5 + z * r;
    r = 0x1.1111111111111p-4 + z * r;
    r = 0x1.3b13b13b13b14p-4 + z * r;
    r = 0x1.745d1745d1746p-4 + z * r;
    r = 0x1.c71c71c71c71cp-4 + z * r;
    r = 0x1.2492492492492p-3 + z * r;
    r = 0x1.999999999999ap-3 + z * r;
    r = 0x1.5555555555555p-2 + z * r;
    double ls = 2.0 * s;
    double lm = ls + (ls * z) * r;
    double de = (double)e;
    return (de * 0x1.a39ef35793c76p-33 + lm) + de * 0x1.62e42fee00000p-1;
}

#if defined(__CUDACC__)
// Exact f32 -> f64 widening built on the integer pipe. GB300's FP64 pipe limits the FP64 channel
// kernel, and the 72 widenings of a step's field gathers would otherwise take a fifth of its FP64
// instructions (measured: 14-19% faster, bit-identical states). Normal numbers and zeros are
// assembled from their bits (exponent rebased by 1023 - 127, the 23-bit fraction moved to the top
// of the 52-bit one); subnormals, infinities and NaN take the hardware conversion. Either way the
// value is the same double (checked against the hardware conversion on 6e8 bit patterns).
__device__ __forceinline__ double widen(float f) {
    const uint32_t u = __float_as_uint(f);
    const uint32_t e = (u >> 23) & 0xFFu;
    if (e - 1u >= 0xFEu && (u & 0x7FFFFFFFu) != 0u) return (double)f;
    const uint32_t sign = u & 0x80000000u;
    const uint32_t hi = (u & 0x7FFFFFFFu) ? (sign | ((e + 896u) << 20) | ((u & 0x7FFFFFu) >> 3)) : sign;
    return __hiloint2double((int)hi, (int)(u << 29));
}

// x / h correctly rounded without a division (h > 0, inv_h = RN(1/h)): q = x * inv_h, then one
// step of Markstein's correction q + (x - q h) inv_h with fused multiply-adds (P. Markstein, IBM J.
// Res. Dev. 34 (1990) 111-119: with a correctly rounded reciprocal and a quotient within one ulp,
// the corrected quotient is the correctly rounded one, barring overflow and underflow, which
// positions and grid spacings never reach). The sign of a zero quotient is the dividend's, as in
// x / h with h > 0. Three FP64 operations in place of the division's sequence on GB300's narrow
// FP64 pipe; checked against IEEE x / h on 2.1e9 positions at 14 grid spacings, and bit for bit
// by the oracle parity tests of both FP64 kernels.
__device__ __forceinline__ double div_rn(double x, double h, double inv_h) {
    const double q = __dmul_rn(x, inv_h);
    return copysign(fma(fma(-q, h, x), inv_h, q), x);
}
#endif

// ---------------------------------------------------------------- random numbers (world.rs:386-402)
MQ_HD uint64_t splitmix(uint64_t z) {
    z = z + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
MQ_HD double xs_next(uint64_t* st) {
    uint64_t x = *st;
    x ^= x << 13;
    x ^= x >> 7;
    x ^= x << 17;
    *st = x;
    return (double)(x >> 11) / 9007199254740992.0;
}
MQ_HD double gauss(double u1, double u2) {
    double s, c;
    sincos2pi(u2, &s, &c);
    return sqrt(-2.0 * log_(u1 > 1e-300 ? u1 : 1e-300)) * c;
}

// ---------------------------------------------------------------- per-batch / per-job constants

struct Batch {             // batch_params (channel.rs:397-410) in f64
    double dt, v_rf, w_rf, h;
    double z_return, z_exit, crash_z0, crash_z1;
    double lim[3];
    double a, z_inject, r_inject, sigma;
    int32_t nx, ny, nz;
    uint32_t max_steps;
    int32_t nearest, legacy_coll, launch, rf_phase0;
};

struct JobC {              // job_params (channel.rs:412-426) in f64
    double qmdt, v_ac, w_ac, nsd, s_gas, mr, floor_v, mfp_mean, s_ion, m, zc;
    int32_t use_ac, tab;
};

// ---------------------------------------------------------------- injection
// Ion::inject (world.rs:407-422) with chsim's legacy launch (channel.rs:350-355) and a
// Gaussian spot; seed = splitmix(job seed + i * 0x9E37) (validate.rs:28).
struct Ion0 {
    double x[3], v[3], ph_rf, ph_ac;
    uint64_t rng;
    int32_t leg;
};

MQ_HD void inject_one(const Batch& b, const JobC& j, uint64_t seed, Ion0* o) {
    uint64_t st = seed | 1ull;
    const double a = b.a, zi = b.z_inject;
    if (b.launch == 1) {
        double kin = 0.1 * (0.75 + 0.75 * xs_next(&st)) * j.zc;
        double vin = sqrt(2.0 * kin * QE / j.m);
        double ang = (-10.0 + 20.0 * xs_next(&st)) * (0x1.921fb54442d18p+1 / 180.0);
        double sa = sin_poly(ang), ca = cos_poly(ang);
        double vx = 0.707 * vin * sa;
        o->x[0] = a; o->x[1] = a; o->x[2] = zi;
        o->v[0] = vx; o->v[1] = vx; o->v[2] = vin * ca;
    } else {
        if (b.launch == 2) {
            double u1 = xs_next(&st), u2 = xs_next(&st);
            o->x[0] = a + b.sigma * gauss(u1, u2);
            u1 = xs_next(&st); u2 = xs_next(&st);
            o->x[1] = a + b.sigma * gauss(u1, u2);
        } else {
            double r = b.r_inject * sqrt(xs_next(&st));
            double s, c;
            sincos2pi(xs_next(&st), &s, &c);
            o->x[0] = a + r * c;
            o->x[1] = a + r * s;
        }
        o->x[2] = zi;
        double u1 = xs_next(&st), u2 = xs_next(&st);
        o->v[0] = j.s_ion * gauss(u1, u2);
        u1 = xs_next(&st); u2 = xs_next(&st);
        o->v[1] = j.s_ion * gauss(u1, u2);
        u1 = xs_next(&st);
        o->v[2] = j.s_ion * sqrt(-2.0 * log_(u1 > 1e-300 ? u1 : 1e-300));
    }
    o->ph_ac = xs_next(&st);
    double prf = xs_next(&st);
    o->ph_rf = b.rf_phase0 ? 0.0 : prf;
    double u = xs_next(&st);
    double first = -log_(u > 1e-7 ? u : 1e-7) * j.mfp_mean / 10.0;   // channel.rs:365-366
    double vmag = sqrt(o->v[0] * o->v[0] + o->v[1] * o->v[1] + o->v[2] * o->v[2]);
    double s0 = floor(first / vmag / b.dt) + 1.0;
    o->leg = !(s0 < 2147483647.0) ? 2147483647 : (int32_t)s0;
    o->rng = st | 1ull;
}

// ---------------------------------------------------------------- drive phase (Clock::fill)
// sin / cos of 2 pi frac(n w) for global step n
MQ_HD void phase_at(double w, uint32_t n, double* s, double* c) {
    double p = (double)n * w;
    sincos2pi(p - floor(p), s, c);
}

MQ_HD int32_t cell_lo(double g, int32_t n) {   // (g.max(0.0) as usize).min(n - 2)
    if (!(g > 0.0)) return 0;
    if (g >= (double)(n - 2)) return n - 2;
    return (int32_t)g;
}
MQ_HD int32_t node_round(double g, int32_t n) {   // ((x / h).round() as usize).min(n - 1)
    double r = round(g);
    if (!(r > 0.0)) return 0;
    if (r >= (double)(n - 1)) return n - 1;
    return (int32_t)r;
}

}  // namespace mqp
