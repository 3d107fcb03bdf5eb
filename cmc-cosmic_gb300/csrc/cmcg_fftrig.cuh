// cmcg_fftrig.cuh -- sine and cosine on the FP32 pipe, in double-float.
//
// The relaxation takes the sine and cosine of three angles per pair: two
// uniform draws times 2 pi (the azimuth of the second star's velocity and the
// deflection's azimuth psi, cmc_dynamics_helper.c:839-849, cmc_dynamics.c:465)
// and the deflection angle beta in [0, pi/2].  Its results are held to 1e-12
// of the reference's, and the kernel is bound by the FP64 pipe.  With
// cmcg_params.relax_trig32 (k_relax64t) they are evaluated here, mostly on the
// FP32 pipe, instead of by FP64 sincos:
//  * reduction to theta in [0, pi/4] by quadrant and complement -- for the
//    uniform angles exactly, on the integer bits of the 32-bit draw (the
//    angle is 2 pi w 2^-32);
//  * Taylor series of sin and cos on [0, pi/4]: the leading terms in
//    double-float arithmetic (a value as an unevaluated sum hi + lo of two
//    floats; products by FMA-based two-product and sums by two-sum, Dekker
//    (1971), "A floating-point technique for extending the available
//    precision", Numer. Math. 18; Knuth, TAOCP vol. 2, 4.2.2), the terms
//    below 2^-40 of the value in float (their float rounding is below
//    2^-64 of it);
//  * truncation after x^15 (sin) and x^16 (cos): the next term is below
//    5e-17 at pi/4.
// Each double-float operation errs by at most ~2^-47 of its result; the
// chains here take about a dozen, so the results are within ~1e-13 of the
// true sine and cosine (tests/test_gpu_parity.py compares them with float64
// sin and cos over the whole range: 2e-14 at most).  Only the conversions of
// the results (and of beta) to and from double use the FP64 pipe.  An ulp-
// accurate sincos keeps a free-running run on the reference's trajectory a
// step longer; so FP64 sincos stays the default.
#pragma once

namespace cmcg {

struct DFl {
    float hi, lo;
};

__device__ __forceinline__ DFl dfl_fast_two_sum(float a, float b)  // |a| >= |b|
{
    const float s = __fadd_rn(a, b);
    return DFl{s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ DFl dfl_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return DFl{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}

__device__ __forceinline__ DFl dfl_mul(DFl a, DFl b)
{
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);  // a.hi b.hi - p exactly
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return dfl_fast_two_sum(p, e);
}

__device__ __forceinline__ DFl dfl_add(DFl a, DFl b)
{
    const DFl s = dfl_two_sum(a.hi, b.hi);
    return dfl_fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}

// c + y x as double-float (one Horner step)
__device__ __forceinline__ DFl dfl_horner(DFl c, DFl y, DFl x) { return dfl_add(c, dfl_mul(y, x)); }

// A double-float constant from its double value: hi the nearest float, lo the
// nearest float to the remainder.
#define CMCG_DFL_CONST(name, v) \
    constexpr float name##_hi = (float)(v), name##_lo = (float)((v) - (double)(float)(v))

CMCG_DFL_CONST(DFL_PIO2, 1.57079632679489661923132169163975144);
CMCG_DFL_CONST(DFL_S3, -1.0 / 6.0);
CMCG_DFL_CONST(DFL_S5, 1.0 / 120.0);
CMCG_DFL_CONST(DFL_S7, -1.0 / 5040.0);
CMCG_DFL_CONST(DFL_C4, 1.0 / 24.0);
CMCG_DFL_CONST(DFL_C6, -1.0 / 720.0);
CMCG_DFL_CONST(DFL_C8, 1.0 / 40320.0);

// sin and cos of theta in [0, pi/4], theta as double-float
__device__ __forceinline__ void dfl_sincos_reduced(DFl x, DFl *s, DFl *c)
{
    const DFl y = dfl_mul(x, x);
    const float yf = y.hi;
    // sin: x (1 - y/3! + y^2/5! - y^3/7! + y^4 T(y)), T in float (x^9 .. x^15)
    float t = -1.0f / 1307674368000.0f;                     // -1/15!
    t = __fmaf_rn(t, yf, 1.0f / 6227020800.0f);             // 1/13!
    t = __fmaf_rn(t, yf, -1.0f / 39916800.0f);              // -1/11!
    t = __fmaf_rn(t, yf, 1.0f / 362880.0f);                 // 1/9!
    DFl a = dfl_horner(DFl{DFL_S7_hi, DFL_S7_lo}, y, DFl{t, 0.0f});
    a = dfl_horner(DFl{DFL_S5_hi, DFL_S5_lo}, y, a);
    a = dfl_horner(DFl{DFL_S3_hi, DFL_S3_lo}, y, a);
    a = dfl_horner(DFl{1.0f, 0.0f}, y, a);
    *s = dfl_mul(x, a);
    // cos: 1 - y/2 + y^2/4! - y^3/6! + y^4/8! + y^5 U(y), U in float (x^10 .. x^16)
    float u = 1.0f / 20922789888000.0f;                     // 1/16!
    u = __fmaf_rn(u, yf, -1.0f / 87178291200.0f);           // -1/14!
    u = __fmaf_rn(u, yf, 1.0f / 479001600.0f);              // 1/12!
    u = __fmaf_rn(u, yf, -1.0f / 3628800.0f);               // -1/10!
    DFl b = dfl_horner(DFl{DFL_C8_hi, DFL_C8_lo}, y, DFl{u, 0.0f});
    b = dfl_horner(DFl{DFL_C6_hi, DFL_C6_lo}, y, b);
    b = dfl_horner(DFl{DFL_C4_hi, DFL_C4_lo}, y, b);
    b = dfl_horner(DFl{-0.5f, 0.0f}, y, b);
    *c = dfl_horner(DFl{1.0f, 0.0f}, y, b);
}

__device__ __forceinline__ double dfl_to_double(DFl a) { return __dadd_rn((double)a.hi, (double)a.lo); }

// sin and cos of 2 pi w 2^-32 for a 32-bit draw w (the angle u01(w) * 2 pi).
__device__ __forceinline__ void sincos_2pi_draw(unsigned int w, double *s, double *c)
{
    const unsigned int q = w >> 30;           // quadrant
    unsigned int f = w & 0x3fffffffu;         // the angle within it: f 2^-30 pi/2
    const bool hi_half = f > 0x20000000u;     // beyond pi/4: its complement
    if (hi_half) f = 0x40000000u - f;
    // f 2^-30 as double-float, exactly: its top 24 bits and its low 6
    const DFl g{__uint2float_rn(f & 0xffffffc0u) * 0x1p-30f, __uint2float_rn(f & 0x3fu) * 0x1p-30f};
    DFl sr, cr;
    dfl_sincos_reduced(dfl_mul(g, DFl{DFL_PIO2_hi, DFL_PIO2_lo}), &sr, &cr);
    double sv = dfl_to_double(hi_half ? cr : sr), cv = dfl_to_double(hi_half ? sr : cr);
    // rotate by the quadrant: (s, c) -> (c, -s) -> (-s, -c) -> (-c, s)
    if (q & 1u) {
        const double t = sv;
        sv = cv;
        cv = -t;
    }
    if (q & 2u) {
        sv = -sv;
        cv = -cv;
    }
    *s = sv;
    *c = cv;
}

// sin and cos of beta in [0, pi/2] (the deflection angle)
__device__ __forceinline__ void sincos_beta(double beta, double *s, double *c)
{
    // below 2^-60 a float would lose beta; sin = beta and cos = 1 there to double
    // precision (beta^3/6 and beta^2/2 are below 2^-120 of them)
    if (__double_as_longlong(beta) < __double_as_longlong(0x1p-60)) {
        *s = beta;
        *c = 1.0;
        return;
    }
    // beyond pi/4: its complement pi/2 - beta (beta >= 0: compared on the bit patterns)
    const bool hi_half = __double_as_longlong(beta) > __double_as_longlong(0.78539816339744830962);
    const double th = hi_half ? __dsub_rn(1.57079632679489661923, beta) : beta;
    const float h = __double2float_rn(th);
    const DFl x{h, __double2float_rn(__dsub_rn(th, (double)h))};
    DFl sr, cr;
    dfl_sincos_reduced(x, &sr, &cr);
    *s = dfl_to_double(hi_half ? cr : sr);
    *c = dfl_to_double(hi_half ? sr : cr);
}

}  // namespace cmcg
