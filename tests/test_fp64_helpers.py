"""The arithmetic shortcuts of the FP64 kernels (csrc/mq_phys.h, csrc/mq_f64.cu), restated in C on
the host and checked against the IEEE operations they replace:

* widen: an f32 widened to f64 by assembling the double's bits equals the hardware conversion
  (every 4099th bit pattern, plus zeros, subnormals, extremes, infinities);
* div_rn: x * RN(1/h) with one Markstein correction by fused multiply-adds equals IEEE x / h
  (2e7 dividends over positions, small and signed values and grid multiples at the spacings the
  engines use, in metres and in millimetres);
* the integer-pipe comparisons and conversions of the channel step: x > c, x < c (c > 0), x < 0,
  the clamped truncation cell_lo and the int -> double conversion agree with the double operations
  on 2e7 values of every sign and exponent, zeros, subnormals, infinities and NaNs.

The GPU parity tests compare the kernels' states with the oracle's bit for bit; these tests pin the
formulas themselves across far more inputs than a trajectory visits."""
import shutil
import subprocess

import pytest

SRC = r"""
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

static double widen(float f) {
    uint32_t u; memcpy(&u, &f, 4);
    const uint32_t e = (u >> 23) & 0xFFu;
    if (e - 1u >= 0xFEu && (u & 0x7FFFFFFFu) != 0u) return (double)f;
    const uint32_t sign = u & 0x80000000u;
    const uint32_t hi = (u & 0x7FFFFFFFu) ? (sign | ((e + 896u) << 20) | ((u & 0x7FFFFFu) >> 3)) : sign;
    const uint64_t b = ((uint64_t)hi << 32) | (uint32_t)(u << 29);
    double d; memcpy(&d, &b, 8); return d;
}
static double div_rn(double x, double h, double inv_h) {
    const double q = x * inv_h;
    return copysign(fma(fma(-q, h, x), inv_h, q), x);
}
typedef long long ll;
static int is_nan_bits(ll b) { return (b & 0x7FFFFFFFFFFFFFFFLL) > 0x7FF0000000000000LL; }
static int gt_pos(ll x, ll c) { return x > c && x <= 0x7FF0000000000000LL; }
static int lt_pos(ll x, ll c) { return x < c && !is_nan_bits(x); }
static int lt_zero(ll x) { return x < 0 && x != (ll)0x8000000000000000ULL && !is_nan_bits(x); }
static ll bits(double d) { ll b; memcpy(&b, &d, 8); return b; }
static int32_t cell_lo(double g, int32_t n) { if (!(g > 0.0)) return 0; if (g >= (double)(n - 2)) return n - 2; return (int32_t)g; }
static int32_t cell_lo_bits(double g, int32_t n, ll lim) {
    const ll b = bits(g);
    if (b <= 0 || b > 0x7FF0000000000000LL) return 0;
    if (b >= lim) return n - 2;
    const int e = (int)(b >> 52) - 1023;
    if (e < 0) return 0;
    return (int32_t)(((b & 0xFFFFFFFFFFFFFLL) | 0x10000000000000LL) >> (52 - e));
}
static double i2d_bits(int32_t v) {
    if (v == 0) return 0.0;
    const int e = 31 - __builtin_clz((unsigned)v);
    const unsigned long long m = ((unsigned long long)(uint32_t)v << (52 - e)) & 0xFFFFFFFFFFFFFULL;
    const unsigned long long b = ((unsigned long long)(1023 + e) << 52) | m;
    double d; memcpy(&d, &b, 8); return d;
}
static uint64_t s = 88172645463325252ull;
static uint64_t xs(void) { s ^= s << 13; s ^= s >> 7; s ^= s << 17; return s; }
static double ud(void) { return (double)(xs() >> 11) * 0x1.0p-53; }

int main(void) {
    unsigned long long bad_w = 0, bad_d = 0, nw = 0, nd = 0;
    const uint32_t special[] = {0u, 0x80000000u, 1u, 0x807fffffu, 0x00800000u, 0x7f7fffffu, 0xff7fffffu,
                                0x7f800000u, 0xff800000u, 0x3f800000u};
    for (uint64_t k = 0; k < (1ull << 32) + sizeof special / 4; ) {
        const uint32_t u = k < (1ull << 32) ? (uint32_t)k : special[k - (1ull << 32)];
        float f; memcpy(&f, &u, 4);
        const double a = widen(f), b = (double)f;
        if (memcmp(&a, &b, 8) != 0) ++bad_w;
        ++nw;
        if (k < (1ull << 32)) { k += 4099; if (k >= (1ull << 32)) k = 1ull << 32; } else ++k;
    }
    const double hs[] = {1e-4, 5e-5, 1e-4 / 3.0, 4e-4, 2e-4, 0.05e-3, 0.51875, 1.0375, 0.5};
    for (unsigned j = 0; j < sizeof hs / sizeof hs[0]; ++j) {
        const double h = hs[j], inv = 1.0 / h, scale = h > 0.1 ? 1000.0 : 1.0;
        for (long i = 0; i < 2200000L; ++i) {
            double x;
            switch (xs() & 3) {
                case 0: x = ud() * 0.05 * scale; break;
                case 1: x = (ud() - 0.5) * 1e-3 * scale; break;
                case 2: x = ldexp(ud() + 0.5, (int)(xs() % 40) - 45); break;
                default: {
                    x = h * (double)(xs() % 2000);
                    uint64_t b; memcpy(&b, &x, 8);
                    if (b > 4) b += (int64_t)(xs() % 5) - 2;
                    memcpy(&x, &b, 8);
                }
            }
            const double a = div_rn(x, h, inv), b = x / h;
            if (memcmp(&a, &b, 8) != 0) ++bad_d;
            ++nd;
        }
        const double z = -0.0, a = div_rn(z, h, inv), b = z / h;
        if (memcmp(&a, &b, 8) != 0) ++bad_d;
    }
    unsigned long long nc = 0, bad_c = 0;
    const double cs[] = {0.5e-3, 1e-3, 23.7e-3, 18.6e-3, 0.0159, 0.0241, 1e-300, 5e-324, 1e300};
    const int32_t ns[] = {2, 3, 160, 242, 480, 726, 1 << 20, 2147483647};
    const double sp[] = {0.0, -0.0, 1.0 / 0.0, -1.0 / 0.0, 0.0 / 0.0, -(0.0 / 0.0), 5e-324, -5e-324, 0.5e-3, 23.7e-3};
    for (long i = 0; i < 20000000L; ++i) {
        double x;
        uint64_t r = xs();
        if ((r & 15) == 0) x = sp[(r >> 4) % (sizeof sp / sizeof sp[0])];
        else if ((r & 15) < 6) { uint64_t b = xs(); memcpy(&x, &b, 8); }           /* any bit pattern */
        else if ((r & 15) < 11) x = (ud() - 0.25) * 0.05;                          /* positions */
        else x = (ud() - 0.1) * (double)(1 << (r >> 8) % 24);                      /* grid units */
        const ll b = bits(x);
        const double c = cs[(r >> 20) % (sizeof cs / sizeof cs[0])];
        const int32_t n = ns[(r >> 28) % (sizeof ns / sizeof ns[0])];
        if (gt_pos(b, bits(c)) != (x > c)) ++bad_c;
        if (lt_pos(b, bits(c)) != (x < c)) ++bad_c;
        if (lt_zero(b) != (x < 0.0)) ++bad_c;
        if (cell_lo_bits(x, n, bits((double)(n - 2))) != cell_lo(x, n)) ++bad_c;
        const int32_t v = (int32_t)(xs() & 0x7FFFFFFF) >> (xs() % 31);
        const double a = i2d_bits(v), d = (double)v;
        if (memcmp(&a, &d, 8) != 0) ++bad_c;
        ++nc;
    }
    printf("%llu %llu %llu %llu %llu %llu\n", nw, bad_w, nd, bad_d, nc, bad_c);
    return 0;
}
"""


def test_fp64_kernel_shortcuts_equal_ieee(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "helpers.c"
    src.write_text(SRC)
    exe = tmp_path / "helpers"
    subprocess.run([cc, "-O2", "-ffp-contract=off", str(src), "-o", str(exe), "-lm"], check=True,
                   capture_output=True, text=True)
    nw, bad_w, nd, bad_d, nc, bad_c = map(int, subprocess.run([str(exe)], check=True, capture_output=True,
                                                           text=True, timeout=120).stdout.split())
    assert nw > 1_000_000 and bad_w == 0, (nw, bad_w)
    assert nd > 19_000_000 and bad_d == 0, (nd, bad_d)
    assert nc == 20_000_000 and bad_c == 0, (nc, bad_c)
