"""The FP64 kernels divide a static row's back substitution by its kept D'
through the correctly rounded reciprocal y = RN(1/D') and Markstein's
correction: q = RN(r*y), e = r - D'*q (exact with one FMA), RN(q + e*y) =
RN(r/D'). This checks the identity on the host's IEEE binary64 arithmetic
(C's division and fma) over random operands and significands next to powers
of two; the GPU parity tests check the kernels' results bit for bit."""
import os
import shutil
import subprocess

import pytest

SRC = r"""
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>
static uint64_t s = 0x9e3779b97f4a7c15ull;
static uint64_t rnd(void) { s ^= s << 13; s ^= s >> 7; s ^= s << 17; return s; }
static double mk(uint64_t mant, int e, int neg)
{
    uint64_t bits = ((uint64_t)(neg ? 1 : 0) << 63) | ((uint64_t)(e + 1023) << 52) | (mant & 0xfffffffffffffull);
    double d;
    memcpy(&d, &bits, 8);
    return d;
}
int main(void)
{
    long long bad = 0;
    for (long long i = 0; i < 2000000LL; ++i) {
        const uint64_t r = rnd();
        uint64_t ma = rnd(), mb = rnd();
        const int kind = (int)(r & 7);
        if (kind == 1) mb = 0xfffffffffffffull - (rnd() & 0xff);
        if (kind == 2) mb = rnd() & 0xff;
        if (kind == 3) ma = 0xfffffffffffffull - (rnd() & 0xff);
        if (kind == 4) ma = rnd() & 0xff;
        const int ea = (int)((r >> 8) % 120) - 60, eb = (int)((r >> 16) % 120) - 60;
        const double a = mk(ma, ea, (r >> 24) & 1), b = mk(mb, eb, (r >> 25) & 1);
        const double y = 1.0 / b;
        const double q = a * y;
        const double q2 = fma(fma(-b, q, a), y, q);
        const double ref = a / b;
        if (memcmp(&q2, &ref, 8) != 0) ++bad;
    }
    printf("%lld\n", bad);
    return 0;
}
"""


def test_markstein_correction_equals_ieee_division(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    src = tmp_path / "div.c"
    exe = tmp_path / "div"
    src.write_text(SRC)
    # no contraction: every product and sum rounds as written; fma() is libm's, correctly rounded
    subprocess.run([cc, "-O2", "-ffp-contract=off", str(src), "-o", str(exe), "-lm"], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True, timeout=120).stdout
    assert int(out.strip()) == 0
