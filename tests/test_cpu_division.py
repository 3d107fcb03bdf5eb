"""The reciprocal-based division the kernels use instead of FP64 division
(div_rcp in cmcg_internal.cuh): restated in C with fma() and compared with
IEEE division, bit for bit, on random and structured operands."""
import os
import subprocess

import pytest

SRC = r"""
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
static uint64_t s[4] = {0x9E3779B97F4A7C15ull, 0xBF58476D1CE4E5B9ull, 0x94D049BB133111EBull, 0x2545F4914F6CDD1Dull};
static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
static uint64_t nxt(void) {
    const uint64_t r = rotl(s[1] * 5, 7) * 9, t = s[1] << 17;
    s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3]; s[2] ^= t; s[3] = rotl(s[3], 45);
    return r;
}
static double mk(uint64_t mant, int e) {
    uint64_t b = ((uint64_t)(e + 1023) << 52) | (mant & ((1ull << 52) - 1));
    double d; memcpy(&d, &b, 8); return d;
}
/* div_rcp: q0 = RN(a y); two corrections q <- RN(q + RN(a - b q) y) */
static double div_rcp(double a, double b, double y) {
    double q0 = a * y;
    double q1 = fma(fma(-q0, b, a), y, q0);
    return fma(fma(-q1, b, a), y, q1);
}
int main(int argc, char **argv) {
    long n = atol(argv[1]), bad = 0;
    for (long i = 0; i < n; i++) {
        uint64_t u = nxt(), v = nxt(), w = nxt();
        uint64_t ma = u, mb = v;
        switch (w & 7) {
        case 1: ma |= ((1ull << 52) - 1) ^ ((w >> 20) & 0xff); break;   /* runs of ones */
        case 2: mb |= ((1ull << 52) - 1) ^ ((w >> 28) & 0xff); break;
        case 3: ma &= ~((1ull << 40) - 1); mb &= ~((1ull << 44) - 1); break;  /* short mantissas */
        case 4: mb = (w >> 12) & 0xffff; break;                        /* b near a power of two */
        case 5: ma = ((1ull << 52) - 1) - ((w >> 13) & 0xfff); break;
        case 6: ma = mb ^ ((w >> 9) & 0x3ff); break;                  /* a/b near 1 */
        }
        double a = mk(ma, (int)((w >> 40) % 400) - 200), b = mk(mb, (int)((w >> 48) % 400) - 200);
        if (w >> 63) a = -a;
        if ((w >> 62) & 1) b = -b;
        double y = 1.0 / b;
        if (div_rcp(a, b, y) != a / b) {
            if (++bad < 4) printf("mismatch a=%a b=%a\n", a, b);
        }
    }
    printf("%ld of %ld differ\n", bad, n);
    return bad != 0;
}
"""


def test_reciprocal_division_is_correctly_rounded(tmp_path):
    src = tmp_path / "divrcp.c"
    src.write_text(SRC)
    exe = tmp_path / "divrcp"
    # -ffp-contract=off: the products and sums round exactly as written
    subprocess.run(["gcc", "-O2", "-ffp-contract=off", str(src), "-o", str(exe), "-lm"], check=True)
    res = subprocess.run([str(exe), "20000000"], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout
