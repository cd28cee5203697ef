// Double-FP32 ("pair") arithmetic on the FP32 pipes, shared by the
// FP64-accurate products, the far M2L evaluated from the points and the
// pivot search for the kernels built on log.
//
// A value is an unevaluated pair of floats (hi + lo, about 2^-48 relative)
// and every operation an error-free transformation: TwoSum (Knuth),
// TwoProduct with the FMA (Ogita, Rump and Oishi 2005), the pair arithmetic
// of Dekker (1971). log(R^2) follows Tang's table-driven method (ACM TOMS
// 16(4), 1990): R^2 = 2^e m, m in [1, 2), c_k the centre of the 1/128-wide
// bin of m (exact in FP32), log m = log c_k + log(1 + u) with u = (m - c_k) /
// c_k, |u| <= 2^-8, log c_k and 1 / c_k from a table of pairs computed on the
// host in FP64, and log(1 + u) = u - u^2/2 + u^3 (1/3 - u/4 + u^2/5) (the u^6
// term is below 2^-50); e log 2 with log 2 split so that e * hi is exact.
#pragma once
#include <cuda_runtime.h>

namespace h2w {

struct Df { float h, l; };
__device__ __forceinline__ Df df_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b), bb = __fsub_rn(s, a);
    return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ Df df_fast(float a, float b) {  // |a| >= |b|
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ Df df_add(Df a, Df b) {
    const Df s = df_two_sum(a.h, b.h);
    return df_fast(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ Df df_sub(Df a, Df b) { return df_add(a, Df{-b.h, -b.l}); }
// (a.h + a.l)^2, not renormalised: hi and a correction below 2^-22 |hi|
__device__ __forceinline__ Df df_sqr(Df a) {
    const float p = __fmul_rn(a.h, a.h);
    return {p, __fmaf_rn(__fadd_rn(a.h, a.h), a.l, __fmaf_rn(a.h, a.h, -p))};
}
__device__ __forceinline__ Df df_mul(Df a, Df b) {
    const float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    return df_fast(p, e);
}

struct DfLogTab { float c, lh, ll, ih, il, pad0, pad1, pad2; };  // bin centre, log c (pair), 1/c (pair)

// log(R^2) as a pair, R^2 = r.h + r.l > 0 and normal
__device__ __forceinline__ Df df_log(Df r, const DfLogTab *tab) {
    const int bits = __float_as_int(r.h);
    const int e = (bits >> 23) - 127;
    const int k = (bits >> 16) & 0x7f;
    const float m = __int_as_float((bits & 0x7fffff) | 0x3f800000);
    const DfLogTab t = tab[k];
    const float d = __fsub_rn(m, t.c);                                   // exact (Sterbenz)
    const float lm = __fmul_rn(r.l, __int_as_float((127 - e) << 23));   // r.l / 2^e, exact
    const Df dd = df_two_sum(d, lm);
    // u = dd / c as a pair
    const float uh = __fmul_rn(dd.h, t.ih);
    float ue = __fmaf_rn(dd.h, t.ih, -uh);
    ue = __fmaf_rn(dd.h, t.il, ue);
    ue = __fmaf_rn(dd.l, t.ih, ue);
    const Df u = df_fast(uh, ue);
    // log(1 + u) = u - u^2/2 + u^3 (1/3 - u/4 + u^2/5)
    const Df u2 = df_sqr(u);
    const float poly = __fmaf_rn(u.h, __fmaf_rn(u.h, 0.2f, -0.25f), 0.33333334f);
    const float tail = __fmul_rn(__fmul_rn(u2.h, u.h), poly);
    Df l1 = df_add(u, Df{-0.5f * u2.h, __fmaf_rn(-0.5f, u2.l, tail)});
    // + e log 2 (hi exact for |e| < 128) + log c
    const float ln2h = 0.693145751953125f, ln2l = 1.42860676533018704e-6f;
    const Df el = df_fast(__fmul_rn((float)e, ln2h), __fmul_rn((float)e, ln2l));
    const Df lc = Df{t.lh, t.ll};
    return df_add(df_add(el, lc), l1);
}

// A double as a pair: hi = fl32(a), lo = fl32(a - hi) (FP64 instructions).
__device__ __forceinline__ float2 df_split(double a) {
    const float h = __double2float_rn(a);
    return make_float2(h, __double2float_rn(__dsub_rn(a, (double)h)));
}
// The same pair without FP64 instructions (GB300 runs those at 1/64 rate):
// hi = the double's top 24 significand bits as a float (truncated), lo = the
// remaining 29 bits, converted to float (rounded to 24 bits) and scaled by the
// exact power of two 2^(E-52); hi + lo carries 47 bits. Used when both parts
// are normal floats (exponent E in [-74, 127]); otherwise (zero, tiny or huge
// values) the FP64 split.
__device__ __forceinline__ float2 df_split_fast(double a) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(a);
    const int e = (int)((u >> 52) & 0x7ff);
    if (e < 1023 - 74 || e > 1023 + 127) return df_split(a);
    const unsigned sign = (unsigned)(u >> 63) << 31;
    const float hi = __uint_as_float(sign | ((unsigned)(e - 1023 + 127) << 23) | (unsigned)((u >> 29) & 0x7fffffu));
    const float scale = __uint_as_float((unsigned)(e - 1023 - 52 + 127) << 23);
    const float lo = __fmul_rn(__uint2float_rn((unsigned)(u & 0x1fffffffu)), scale);
    return make_float2(hi, sign ? -lo : lo);
}

}  // namespace h2w
