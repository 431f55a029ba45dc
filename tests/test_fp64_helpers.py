"""The two arithmetic shortcuts of the FP64 kernels (csrc/mq_phys.h), restated in C on the host and
checked against the IEEE operations they replace:

* widen: an f32 widened to f64 by assembling the double's bits equals the hardware conversion
  (every 4099th bit pattern, plus zeros, subnormals, extremes, infinities);
* div_rn: x * RN(1/h) with one Markstein correction by fused multiply-adds equals IEEE x / h
  (2e7 dividends over positions, small and signed values and grid multiples at the spacings the
  engines use, in metres and in millimetres).

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
    printf("%llu %llu %llu %llu\n", nw, bad_w, nd, bad_d);
    return 0;
}
"""


def test_widen_and_markstein_division(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "helpers.c"
    src.write_text(SRC)
    exe = tmp_path / "helpers"
    subprocess.run([cc, "-O2", "-ffp-contract=off", str(src), "-o", str(exe), "-lm"], check=True,
                   capture_output=True, text=True)
    nw, bad_w, nd, bad_d = map(int, subprocess.run([str(exe)], check=True, capture_output=True,
                                                   text=True, timeout=120).stdout.split())
    assert nw > 1_000_000 and bad_w == 0, (nw, bad_w)
    assert nd > 19_000_000 and bad_d == 0, (nd, bad_d)
