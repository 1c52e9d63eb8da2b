// f32x2.cuh -- two-float arithmetic (a value held as the unevaluated sum
// h + l of two floats, about 48 significant bits) and the increments of the
// Langevin step (src/bin/simulation/mod.rs:318-369) computed in it: the
// canonical quasi-2-D chain (langevin_canon in common.cuh) and the full
// chain (langevin<> in common.cuh, 3-D and quasi-2-D rows off the canonical
// state).
//
// GB300 issues FP32 at 128 operations per clock per SM and FP64 at 2, so a
// two-float operation of 3 to 11 FP32 instructions costs a fraction of one
// FP64 instruction.  The particle state stays FP64.  A step's increments
// (dx, dy of order |v| dt + sqrt(2 Dt dt) |xi|, the angle changes of order
// |rot|) are small beside the coordinates they are added to, so their
// relative error of about 2^-47 lies near or below an ulp of the new
// coordinate; those additions (two per coordinate, h then l) are the only
// FP64 arithmetic.
//
// Error-free transformations (Dekker 1971; Knuth, TAOCP vol. 2, 4.2.2;
// Muller et al., Handbook of Floating-Point Arithmetic, ch. 4): two_sum,
// fast_two_sum and two_prod with a fused multiply-add.  On the device every
// FP32 operation carries an explicit rounding intrinsic, so the compiler
// neither contracts nor reorders them; a host build (the CPU tests compile
// this header with g++) needs -ffp-contract=off.
#pragma once

#include <stdint.h>

#ifdef __CUDACC__
#define SS_XF __device__ __forceinline__
#define SS_TRIGF_ATTR static __device__
#else
#include <math.h>
#include <string.h>
#define SS_XF static inline
#define SS_TRIGF_ATTR static const
struct float4 {
    float x, y, z, w;
};
struct float2 {
    float x, y;
};
#endif

namespace ss {
namespace xf {

#include "trig_table_f.inc"

struct f2 {
    float h, l;
};

// ---- rounding-exact primitives and bit casts ---------------------------
#ifdef __CUDA_ARCH__
SS_XF float add_(float a, float b) { return __fadd_rn(a, b); }
SS_XF float sub_(float a, float b) { return __fsub_rn(a, b); }
SS_XF float mul_(float a, float b) { return __fmul_rn(a, b); }
SS_XF float fma_(float a, float b, float c) { return __fmaf_rn(a, b, c); }
SS_XF float rcp_(float a) { return __frcp_rn(a); }
SS_XF float fdiv_approx(float a, float b) { return __fdividef(a, b); }
SS_XF float i2f_(int i) { return __int2float_rn(i); }
SS_XF long long dbits(double d) { return __double_as_longlong(d); }
SS_XF double bitsd(long long b) { return __longlong_as_double(b); }
SS_XF uint32_t fbits(float f) { return __float_as_uint(f); }
SS_XF float bitsf(uint32_t u) { return __uint_as_float(u); }
SS_XF int clz32(uint32_t v) { return __clz((int)v); }
SS_XF float4 trigf(int j) { return __ldg(&kTrigF[j]); }
SS_XF float2 ldg2(const float2 *p) { return __ldg(p); }
SS_XF double atan2_(double y, double x) { return atan2(y, x); }
SS_XF void sincos_(double a, double *s, double *c) { sincos(a, s, c); }
#else
SS_XF float add_(float a, float b) { return a + b; }
SS_XF float sub_(float a, float b) { return a - b; }
SS_XF float mul_(float a, float b) { return a * b; }
SS_XF float fma_(float a, float b, float c) { return fmaf(a, b, c); }
SS_XF float rcp_(float a) { return 1.0f / a; }
SS_XF float fdiv_approx(float a, float b) { return a / b; }
SS_XF float i2f_(int i) { return (float)i; }
SS_XF long long dbits(double d) { long long b; memcpy(&b, &d, 8); return b; }
SS_XF double bitsd(long long b) { double d; memcpy(&d, &b, 8); return d; }
SS_XF uint32_t fbits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
SS_XF float bitsf(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
SS_XF int clz32(uint32_t v) { return v ? __builtin_clz(v) : 32; }
SS_XF float4 trigf(int j) { return kTrigF[j]; }
SS_XF float2 ldg2(const float2 *p) { return *p; }
SS_XF double atan2_(double y, double x) { return atan2(y, x); }
SS_XF void sincos_(double a, double *s, double *c) { *s = sin(a); *c = cos(a); }
#endif

// s + e = a + b exactly
SS_XF f2 two_sum(float a, float b) {
    const float s = add_(a, b), bb = sub_(s, a);
    return {s, add_(sub_(a, sub_(s, bb)), sub_(b, bb))};
}
// s + e = a + b exactly when |a| >= |b| or a == 0
SS_XF f2 fast_two_sum(float a, float b) {
    const float s = add_(a, b);
    return {s, sub_(b, sub_(s, a))};
}
// p + e = a b exactly
SS_XF f2 two_prod(float a, float b) {
    const float p = mul_(a, b);
    return {p, fma_(a, b, -p)};
}
SS_XF f2 neg(f2 a) { return {-a.h, -a.l}; }
// a + b, absolute error about 2^-47 (|a| + |b|)
SS_XF f2 add(f2 a, f2 b) {
    const f2 s = two_sum(a.h, b.h);
    return fast_two_sum(s.h, add_(s.l, add_(a.l, b.l)));
}
// a b, relative error about 2^-46
SS_XF f2 mul(f2 a, f2 b) {
    const f2 p = two_prod(a.h, b.h);
    return fast_two_sum(p.h, fma_(a.h, b.l, fma_(a.l, b.h, p.l)));
}
SS_XF f2 mul(f2 a, float b) {
    const f2 p = two_prod(a.h, b);
    return fast_two_sum(p.h, fma_(a.l, b, p.l));
}
// a b as an unnormalised pair (|l| up to a few ulps of h), for a sum that
// normalises next
SS_XF f2 mul_u(f2 a, f2 b) {
    const f2 p = two_prod(a.h, b.h);
    return {p.h, fma_(a.h, b.l, fma_(a.l, b.h, p.l))};
}
SS_XF f2 mul_u(f2 a, float b) {
    const f2 p = two_prod(a.h, b);
    return {p.h, fma_(a.l, b, p.l)};
}
// a b as an unnormalised pair (|l| up to a few ulps of h)
SS_XF f2 prod(float ah, float al, f2 b) {
    const f2 p = two_prod(ah, b.h);
    return {p.h, fma_(ah, b.l, fma_(al, b.h, p.l))};
}

// ---- conversions from a double's bits (no FP64 instruction) -----------
// the exact double of a float (zero, subnormals, inf and NaN included)
SS_XF double to_double(float f) {
    const uint32_t u = fbits(f);
    const uint32_t a = u & 0x7FFFFFFFu;
    if (a - 0x00800000u < 0x7F000000u)  // normal (exponent field 1 .. 254): (e + 896) << 52 | m << 29
        return bitsd((long long)((((unsigned long long)a << 29) + (896ull << 52)) |
                                 ((unsigned long long)(u & 0x80000000u) << 32)));
    const uint32_t e = (u >> 23) & 0xFFu, m = u & 0x7FFFFFu;
    unsigned long long body;
    if (e == 0xFFu) {
        body = (0x7FFull << 52) | ((unsigned long long)m << 29);
    } else if (e != 0u) {
        body = ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)m << 29);
    } else if (m == 0u) {
        body = 0ull;
    } else {  // m 2^-149 with the highest set bit p of m
        const int p = 31 - clz32(m);
        body = ((unsigned long long)(p + 874) << 52) | (((unsigned long long)m << (52 - p)) & 0xFFFFFFFFFFFFFull);
    }
    return bitsd((long long)(((unsigned long long)(u & 0x80000000u) << 32) | body));
}

// The pair nearest a double d: h = d rounded to float (ties to even), l =
// d - h rounded to float.  |d| < 2^-126 gives (0, 0) (with d's sign);
// |d| >= 2^128, infinities and NaN give (+-inf or NaN, 0).
SS_XF f2 split(double d) {
    const unsigned long long b = (unsigned long long)dbits(d);
    const uint32_t sgn = (uint32_t)(b >> 32) & 0x80000000u;
    const int e = (int)((b >> 52) & 0x7FFu);
    if (e < 1023 - 126) return {bitsf(sgn), 0.0f};
    if (e >= 1023 + 128) {
        const bool nan = e == 0x7FF && (b & 0xFFFFFFFFFFFFFull);
        return {bitsf(sgn | (nan ? 0x7FC00000u : 0x7F800000u)), 0.0f};
    }
    const unsigned long long m = b & 0xFFFFFFFFFFFFFull;
    uint32_t f = ((uint32_t)(e - 896) << 23) | (uint32_t)(m >> 29);
    int rest = (int)(m & 0x1FFFFFFFull);  // the 29 bits below h's last
    if (rest > 0x10000000 || (rest == 0x10000000 && (f & 1u))) {
        f += 1u;  // a carry into the exponent field is the correct rounding
        rest -= 0x20000000;
    }
    const float h = bitsf(sgn | f);
    if (rest == 0) return {h, 0.0f};
    // l = rest 2^(e - 1075) with d's sign: rest as a float (rounded when it
    // has more than 24 bits), its exponent lowered by 1075 - e
    const float r = i2f_(rest);
    const int er = (int)((fbits(r) >> 23) & 0xFFu) - (1075 - e);
    if (er < 1) return {h, 0.0f};  // below 2^-126: dropped (d below 2^-97)
    return {h, bitsf(((fbits(r) & 0x807FFFFFu) ^ sgn) | ((uint32_t)er << 23))};
}

// ---- sin and cos from the table of j / 512 -----------------------------
// kTrigF[j] = (cos a_j, sin a_j) at a_j = j / 512 as pairs (hi, lo).  For
// a = a_j + b, |b| <= 2^-10 (+ a float ulp): sin b = b - b^3/6 + b^5/120 and
// cos b - 1 = -b^2/2 + b^4/24 (omitted terms below 2e-25 and 2e-21); b^2 is
// carried as a pair, the terms b^3/6 <= 1.6e-10 and b^4/24 in FP32 (their
// rounding below 3e-17 absolute).  Then sin a = S + (C sb + S cb) and
// cos a = C + (C cb - S sb), summed with exact two_sums and one rounding of
// the low parts: within about 2^-47 (7e-15) of the exact values.
SS_XF void sincos_red(int j, f2 b, f2 &s, f2 &c) {
    const float4 t = trigf(j);  // (cos hi, cos lo, sin hi, sin lo)
    f2 z = two_prod(b.h, b.h);
    z.l = fma_(add_(b.h, b.h), b.l, z.l);
    const f2 sb = {b.h, add_(b.l, mul_(mul_(b.h, z.h), fma_(z.h, 1.0f / 120.0f, -1.0f / 6.0f)))};
    const f2 cb = {mul_(z.h, -0.5f), fma_(mul_(z.h, z.h), 1.0f / 24.0f, mul_(z.l, -0.5f))};
    {
        const f2 p = prod(t.x, t.y, sb), q = prod(t.z, t.w, cb);
        const f2 u = two_sum(t.z, p.h), v = two_sum(u.h, q.h);
        s = fast_two_sum(v.h, add_(add_(add_(p.l, q.l), add_(u.l, v.l)), t.w));
    }
    {
        const f2 p = prod(t.x, t.y, cb), q = prod(-t.z, -t.w, sb);
        const f2 u = two_sum(t.x, q.h), v = two_sum(u.h, p.h);
        c = fast_two_sum(v.h, add_(add_(add_(p.l, q.l), add_(u.l, v.l)), t.y));
    }
}

// j = round(512 a) for +0 <= a < 6.3, from a's bits; -1 for other a
// (negative, -0.0, larger, NaN)
SS_XF int round512(double a) {
    const long long bits = dbits(a);
    if (bits < 0 || bits >= kTrigFMaxKey) return -1;
    const int e = (int)(bits >> 52) - 1023;
    if (e < -11) return 0;  // a < 2^-11: 512 a < 1/4
    const unsigned long long mant = (unsigned long long)(bits & 0xFFFFFFFFFFFFFll) | (1ull << 52);
    const int shift = 43 - e;  // 512 a = mant 2^-shift, shift in 41 .. 54
    return (int)((mant + (1ull << (shift - 1))) >> shift);
}

// a_j = j / 512 as a double, from j's bits (0 <= j < 2^20)
SS_XF double angle512(int j) {
    if (j == 0) return 0.0;
    const int hb = 31 - clz32((uint32_t)j);
    const unsigned long long b = ((unsigned long long)(1023 + hb - 9) << 52) |
                                 (((unsigned long long)j << (52 - hb)) & 0xFFFFFFFFFFFFFull);
    return bitsd((long long)b);
}

// sin a and cos a of a double angle (the one FP64 instruction: the exact
// reduction a - a_j); angles outside [0, 6.3) take FP64 sincos
SS_XF void sincos_d(double a, f2 &s, f2 &c) {
    const int j = round512(a);
    if (j < 0) {
        double sd, cd;
        sincos_(a, &sd, &cd);
        s = split(sd);
        c = split(cd);
        return;
    }
    sincos_red(j, split(a - angle512(j)), s, c);
}

// round(512 a) for 0 <= a < 2^21 in FP32: adding 1.5 2^23 rounds to an
// integer (ties to even), read from the sum's low mantissa bits
SS_XF int round512f(float a, float &aj) {
    const float big = 12582912.0f;  // 1.5 2^23
    const float t = add_(mul_(a, 512.0f), big);
    aj = mul_(sub_(t, big), 1.0f / 512.0f);  // exact: an integer below 2^21 over 512
    return (int)(fbits(t) - fbits(big));
}

// sin and cos of a pair angle r = h + l >= 0 (the rotation angle; l may be
// a few ulps of h, unnormalised); h >= 6.25 or NaN takes FP64 sincos
SS_XF void sincos_f2(f2 r, f2 &s, f2 &c) {
    if (!(r.h >= 0.0f && r.h < 6.25f)) {
        double sd, cd;
        sincos_(to_double(r.h) + to_double(r.l), &sd, &cd);
        s = split(sd);
        c = split(cd);
        return;
    }
    float aj;
    const int j = round512f(r.h, aj);
    // r.h - a_j is exact (Sterbenz for j >= 1; r.h itself for j == 0)
    sincos_red(j, two_sum(sub_(r.h, aj), r.l), s, c);
}

// sin r and cos r - 1 of a pair angle r >= 0, the latter without the
// cancellation of cos r - 1: (C_j - 1) + C cb - S sb from the table pair
// of C_j (C_j - 1 formed exactly by two_sum).  Absolute error about 2^-48
// on both (the table pair's own rounding of C_j); r.h >= 6.25 or NaN takes
// FP64 sincos.
SS_XF void sin_cosm1_f2(f2 r, f2 &s, f2 &cm1) {
    if (!(r.h >= 0.0f && r.h < 6.25f)) {
        double sd, cd;
        sincos_(to_double(r.h) + to_double(r.l), &sd, &cd);
        s = split(sd);
        cm1 = split(cd - 1.0);
        return;
    }
    float aj;
    const int j = round512f(r.h, aj);
    const f2 b = two_sum(sub_(r.h, aj), r.l);
    const float4 t = trigf(j);
    f2 z = two_prod(b.h, b.h);
    z.l = fma_(add_(b.h, b.h), b.l, z.l);
    const f2 sb = {b.h, add_(b.l, mul_(mul_(b.h, z.h), fma_(z.h, 1.0f / 120.0f, -1.0f / 6.0f)))};
    const f2 cb = {mul_(z.h, -0.5f), fma_(mul_(z.h, z.h), 1.0f / 24.0f, mul_(z.l, -0.5f))};
    {
        const f2 p = prod(t.x, t.y, sb), q = prod(t.z, t.w, cb);
        const f2 u = two_sum(t.z, p.h), v = two_sum(u.h, q.h);
        s = fast_two_sum(v.h, add_(add_(add_(p.l, q.l), add_(u.l, v.l)), t.w));
    }
    {
        const f2 c0 = two_sum(t.x, -1.0f);  // C_j - 1 (with the table's low part below)
        const f2 p = prod(t.x, t.y, cb), q = prod(-t.z, -t.w, sb);
        const f2 u = two_sum(c0.h, q.h), v = two_sum(u.h, p.h);
        cm1 = fast_two_sum(v.h, add_(add_(add_(p.l, q.l), add_(u.l, v.l)), add_(c0.l, t.y)));
    }
}

// sqrt of a pair x >= 0: the FP32 root y of x.h and one correction with the
// exact remainder x - y^2, relative error about 2^-46; (0, 0) for x.h <= 0
SS_XF f2 sqrt_f2(f2 x) {
    if (!(x.h > 0.0f)) return {0.0f, 0.0f};
#ifdef __CUDA_ARCH__
    const float y = __fsqrt_rn(x.h);
#else
    const float y = sqrtf(x.h);
#endif
    const f2 yy = two_prod(y, y);
    const float r = add_(sub_(sub_(x.h, yy.h), yy.l), x.l);  // x.h - yy.h is exact (Sterbenz)
    return fast_two_sum(y, mul_(r, mul_(0.5f, rcp_(y))));
}

// a / b for pairs with b.h > 0 normal: an FP32 quotient and one correction
// with the exact remainder, relative error about 2^-46
SS_XF f2 div_f2(f2 a, f2 b) {
    const float r = rcp_(b.h);
    const float q1 = mul_(a.h, r);
    const f2 p = two_prod(q1, b.h);
    const float rem = add_(sub_(sub_(a.h, p.h), p.l), sub_(a.l, mul_(q1, b.l)));
    return fast_two_sum(q1, mul_(rem, r));
}

// An estimate of atan2(y, x) for y >= 0 (+0 included) within 1.1e-5: the
// ratio of the smaller to the larger of y and |x| in [0, 1], atan of it by
// the odd polynomial of Abramowitz & Stegun 4.4.47 (|error| <= 1e-5), then
// the octant.  Only the table index comes from it.  y = x = 0 gives NaN.
SS_XF float atan2_est(float y, float x) {
    const float ax = fabsf(x);
    const float t = fdiv_approx(fminf(y, ax), fmaxf(y, ax));
    const float t2 = mul_(t, t);
    float a = mul_(t, fma_(t2, fma_(t2, fma_(t2, fma_(t2, 0.0208351f, -0.0851330f), 0.1801410f), -0.3302995f),
                           0.9998660f));
    if (y > ax) a = sub_(1.57079633f, a);
    if (x < 0.0f) a = sub_(3.14159265f, a);
    return a;
}

// atan2(y, x) of pairs.  An FP32 estimate of the angle of (x, |y|) picks
// a_j = j / 512; the vector rotated by -a_j, (d, e) = (x C + |y| S,
// |y| C - x S), has the small angle eps = atan(e / d), |eps| <= 2^-10 +
// 1.1e-5.  e / d from an FP32 reciprocal and one correction with the exact
// remainder; atan eps = eps - eps^3/3 + eps^5/5 (omitted terms below 1e-22,
// the FP32 cubic and quintic terms rounded below 1e-16 absolute).  The sign
// of y is applied last (atan2 is odd in y).  A rotated vector with d not in
// [2^-60, 2^60) or |e| above d 2^-9 (zero, tiny, huge or non-finite input,
// where the estimate fails) takes FP64 atan2.
SS_XF f2 atan2_f2(f2 y, f2 x) {
    const bool negy = (fbits(y.h) >> 31) != 0u;
    const f2 ay = negy ? neg(y) : y;
    float aj;
    const int j = round512f(atan2_est(ay.h, x.h), aj);  // 0 .. 1609 (NaN: checked below)
    f2 ang;
    if (j >= 0 && j < kTrigFN) {
        const float4 t = trigf(j);
        const f2 C = {t.x, t.y}, S = {t.z, t.w};
        // d only scales eps (its error is relative); e cancels (|e| << |y| C),
        // so its products are normalised first
        const f2 d = add(mul_u(x, C), mul_u(ay, S));
        const f2 e = add(mul(ay, C), neg(mul(x, S)));
        const float ad = fabsf(d.h);
        if (d.h >= 0x1p-60f && d.h < 0x1p60f && fabsf(e.h) <= mul_(ad, 0x1p-9f)) {
            const float r = rcp_(d.h);
            const float q1 = mul_(e.h, r);
            const f2 p = two_prod(q1, d.h);
            // e - q1 d: e.h - p.h is exact (Sterbenz), the rest are small
            const float rem = add_(sub_(sub_(e.h, p.h), p.l), sub_(e.l, mul_(q1, d.l)));
            const f2 eps = fast_two_sum(q1, mul_(rem, r));
            const float z = mul_(eps.h, eps.h);
            const float corr = mul_(mul_(eps.h, z), fma_(z, 1.0f / 5.0f, -1.0f / 3.0f));
            const f2 a = two_sum(aj, eps.h);
            ang = fast_two_sum(a.h, add_(a.l, add_(eps.l, corr)));
            return negy ? neg(ang) : ang;
        }
    }
    return split(atan2_(to_double(y.h) + to_double(y.l), to_double(x.h) + to_double(x.l)));
}

// ---- the canonical quasi-2-D increments -------------------------------
// Which terms of the chain run (Langevin modifiers of the step).
struct CanonTerms {
    bool self_propulsion, convection, trans_diffusion, rot_diffusion, external_field, vorticity, strain;
};

SS_XF f2 mul_noise(f2 a, f2 b) { return mul_u(a, b); }
SS_XF f2 mul_noise(f2 a, float b) { return mul_u(a, b); }

// The increments dx, dy, dphi of the canonical quasi-2-D chain for a
// particle at angle phi (FP64, in [0, 2 pi)) in a cell whose pre-multiplied
// table row is ct = 4 float4 (u0 dt, u1 dt | W01 dt, s E00 | s E01, s E11 |
// diffusion length, 0; each value a pair hi, lo; s = shape dt), with the
// noise xi0, xi1 (normals), sa (sine of the rotation axis angle) and rot
// (rotation angle) as floats or pairs.  The terms in the reference's order:
//   dx = cos phi dt + u0 dt + xi0 diff,  dy = sin phi dt + u1 dt + xi1 diff,
//   G = r dt cos phi + W01 dt + (cos phi f1 - sin phi f0) - sa sin rot,
//   f = s E (cos phi, sin phi),  dphi = atan2(G, cos rot).
template <typename XI, typename SA>
SS_XF void canon_increments(double phi, const float4 *ct, XI xi0, XI xi1, SA sa, f2 rot, const CanonTerms &T,
                            f2 dt, f2 reorient_dt, f2 &dx, f2 &dy, f2 &dphi) {
    f2 sp, cp;
    sincos_d(phi, sp, cp);
    const float4 c0 = ct[0], c1 = ct[1], c2 = ct[2], c3 = ct[3];
    const f2 u0 = {c0.x, c0.y}, u1 = {c0.z, c0.w}, w01 = {c1.x, c1.y}, e00 = {c1.z, c1.w};
    const f2 e01 = {c2.x, c2.y}, e11 = {c2.z, c2.w}, diff = {c3.x, c3.y};
    f2 d0 = {0.0f, 0.0f}, d1 = {0.0f, 0.0f};
    if (T.self_propulsion && T.convection) {
        d0 = add(mul_u(cp, dt), u0);
        d1 = add(mul_u(sp, dt), u1);
    } else if (T.self_propulsion) {
        d0 = mul(cp, dt);
        d1 = mul(sp, dt);
    } else if (T.convection) {
        d0 = u0;
        d1 = u1;
    }
    if (T.trans_diffusion) {
        d0 = add(mul_noise(diff, xi0), d0);
        d1 = add(mul_noise(diff, xi1), d1);
    }
    f2 G = {0.0f, 0.0f};
    if (T.external_field) G = mul(reorient_dt, cp);
    if (T.vorticity) G = T.external_field ? add(G, w01) : w01;
    if (T.strain) {
        const f2 f0 = add(mul_u(e00, cp), mul_u(e01, sp)), f1 = add(mul_u(e01, cp), mul_u(e11, sp));
        G = add(G, add(mul_u(cp, f1), neg(mul_u(sp, f0))));
    }
    f2 C = {1.0f, 0.0f};
    if (T.rot_diffusion) {
        f2 sr;
        sincos_f2(rot, sr, C);
        G = add(G, neg(mul_noise(sr, sa)));
    }
    dx = d0;
    dy = d1;
    dphi = atan2_f2(G, C);
}

// ---- the full chain (3-D, and quasi-2-D rows off the canonical state) ----
// Entries of a per-cell field row written as float pairs (the double table
// row's layout, one pair in each 8 bytes): u[3], W01 W02 W12, E00 E01 E02
// E11 E12 E22, the diffusion length, B[3] (times the dipolar coupling),
// grad B[3][3].
constexpr int R_U = 0, R_W01 = 3, R_W02 = 4, R_W12 = 5, R_E00 = 6, R_E01 = 7, R_E02 = 8, R_E11 = 9,
              R_E12 = 10, R_E22 = 11, R_DIFF = 12, R_B = 13, R_GB = 16;

SS_XF f2 row_f2(const float2 *row, int k) {
    const float2 v = ldg2(row + k);
    return {v.x, v.y};
}

struct FullTerms {
    bool self_propulsion, convection, mdd_force, external_field, mdd_rotation, vorticity, strain, step,
        trans_diffusion, rot_diffusion;
};

// The cosine of the rotation axis angle as the on-device noise defines it:
// sqrt(1 - sa^2) with the sign of the FP32 cosine, sa the FP32 sine.
SS_XF f2 axis_cos(float sa, float ca_f32) {
    const f2 s2 = two_prod(sa, sa);
    const f2 om = two_sum(1.0f, -s2.h);
    const f2 c = sqrt_f2(fast_two_sum(om.h, sub_(om.l, s2.l)));
    return (fbits(ca_f32) >> 31) ? neg(c) : c;
}

// Results of the full chain: the position increments and either the angle
// increments (a = dphi, b = dtheta) or, within 2^-10 of a pole, the direct
// angles (a = phi in (-pi, pi], b = pi/2 - theta).
struct FullOut {
    f2 dp[3], a, b;
    bool direct;
};

// The chain of langevin<> (common.cuh; LangevinBuilder and its modifiers,
// src/integrators/langevin_builder/mod.rs:25-125, modifiers.rs:39-231) in
// pairs, term by term in the same order, for a particle at (phi, theta) in
// a cell whose row is `row` (float pairs), with the noise xi (normals), sa,
// ca (the rotation axis angle) and rot (the rotation angle).
//
// The new orientation v = n + dn is turned into angle increments without
// the cancellation of atan2(v) - (phi, theta): with n the unit vector at
// (phi, theta), |n_xy| = sin theta = st,
//   dphi   = atan2(n0 dn1 - n1 dn0, st^2 + n0 dn0 + n1 dn1)
//   dtheta = atan2(delta ct - dn2 st, |v_xy| st + v2 ct),
//   delta  = |v_xy| - st = (2 (n0 dn0 + n1 dn1) + dn0^2 + dn1^2) / (|v_xy| + st),
// the angle between the horizontal projections and the difference of the
// polar angles (|v_xy| itself from the components of v = n + dn).  Each is about 2^-46 of its own size, where the direct
// angles carry 2^-46 of pi.  Near a pole (st < 2^-10) the direct angles
// atan2(v1, v0) and pi/2 - atan2(v2, |v_xy|) of the reference are used.
template <typename XI, typename SA>
SS_XF void full_increments(double phi, double theta, const float2 *row, XI xi0, XI xi1, XI xi2, SA sa, f2 ca,
                           f2 rot, const FullTerms &T, f2 dt, f2 reorient, f2 shape, f2 drag, FullOut &o) {
    f2 sp, cp, st, ct;
    sincos_d(phi, sp, cp);
    sincos_d(theta, st, ct);
    const f2 n[3] = {mul(st, cp), mul(st, sp), ct};
    const f2 zero = {0.0f, 0.0f};
    f2 dp[3] = {zero, zero, zero}, dn[3] = {zero, zero, zero};
    if (T.self_propulsion) {  // modifiers.rs:39-46
        dp[0] = n[0];
        dp[1] = n[1];
        dp[2] = n[2];
    }
    if (T.convection)  // modifiers.rs:49-56
        for (int k = 0; k < 3; ++k) dp[k] = add(dp[k], row_f2(row, R_U + k));
    if (T.mdd_force) {  // modifiers.rs:59-70: grad B . n * drag
        for (int a = 0; a < 3; ++a) {
            const f2 f = add(add(mul_u(row_f2(row, R_GB + 3 * a), n[0]), mul_u(row_f2(row, R_GB + 3 * a + 1), n[1])),
                             mul_u(row_f2(row, R_GB + 3 * a + 2), n[2]));
            dp[a] = add(dp[a], mul_u(f, drag));
        }
    }
    if (T.external_field) {  // modifiers.rs:103-119: b = (0, r, 0), b - n (n . b)
        const f2 d = mul(n[1], reorient);
        dn[0] = add(dn[0], neg(mul_u(n[0], d)));
        dn[1] = add(dn[1], add(reorient, neg(mul_u(n[1], d))));
        dn[2] = add(dn[2], neg(mul_u(n[2], d)));
    }
    if (T.mdd_rotation) {  // modifiers.rs:172-187: b - n (n . b), b the dipolar field
        const f2 b[3] = {row_f2(row, R_B), row_f2(row, R_B + 1), row_f2(row, R_B + 2)};
        const f2 d = add(add(mul_u(n[0], b[0]), mul_u(n[1], b[1])), mul_u(n[2], b[2]));
        for (int k = 0; k < 3; ++k) dn[k] = add(dn[k], add(b[k], neg(mul_u(n[k], d))));
    }
    if (T.vorticity) {  // modifiers.rs:123-143: -(W n), W antisymmetric
        const f2 w01 = row_f2(row, R_W01), w02 = row_f2(row, R_W02), w12 = row_f2(row, R_W12);
        const f2 f0 = add(mul_u(w01, n[1]), mul_u(w02, n[2]));
        const f2 f1 = add(neg(mul_u(w01, n[0])), mul_u(w12, n[2]));
        const f2 f2v = add(neg(mul_u(w02, n[0])), neg(mul_u(w12, n[1])));
        dn[0] = add(dn[0], neg(f0));
        dn[1] = add(dn[1], neg(f1));
        dn[2] = add(dn[2], neg(f2v));
    }
    if (T.strain) {  // modifiers.rs:147-170: f - n (f . n), f = shape E n
        const f2 e00 = row_f2(row, R_E00), e01 = row_f2(row, R_E01), e02 = row_f2(row, R_E02);
        const f2 e11 = row_f2(row, R_E11), e12 = row_f2(row, R_E12), e22 = row_f2(row, R_E22);
        f2 f[3] = {add(add(mul_u(e00, n[0]), mul_u(e01, n[1])), mul_u(e02, n[2])),
                   add(add(mul_u(e01, n[0]), mul_u(e11, n[1])), mul_u(e12, n[2])),
                   add(add(mul_u(e02, n[0]), mul_u(e12, n[1])), mul_u(e22, n[2]))};
        for (int k = 0; k < 3; ++k) f[k] = mul(f[k], shape);
        const f2 fn = add(add(mul_u(f[0], n[0]), mul_u(f[1], n[1])), mul_u(f[2], n[2]));
        for (int k = 0; k < 3; ++k) dn[k] = add(dn[k], add(f[k], neg(mul_u(n[k], fn))));
    }
    if (T.step) {  // mod.rs:114-119
        for (int k = 0; k < 3; ++k) {
            dp[k] = mul(dp[k], dt);
            dn[k] = mul(dn[k], dt);
        }
    }
    if (T.trans_diffusion) {  // modifiers.rs:86-99
        const f2 diff = row_f2(row, R_DIFF);
        dp[0] = add(dp[0], mul_noise(diff, xi0));
        dp[1] = add(dp[1], mul_noise(diff, xi1));
        dp[2] = add(dp[2], mul_noise(diff, xi2));
    }
    if (T.rot_diffusion) {  // modifiers.rs:199-231, as Rodrigues: n (cos r - 1) + (k x n) sin r
        const f2 ax0 = add(mul_noise(mul(cp, ct), sa), neg(mul_u(ca, sp)));
        const f2 ax1 = add(mul_u(ca, cp), mul_u(mul_noise(ct, sa), sp));
        const f2 ax2 = neg(mul_noise(st, sa));
        f2 sr, cm1;
        sin_cosm1_f2(rot, sr, cm1);
        const f2 k0 = add(mul_u(ax1, n[2]), neg(mul_u(ax2, n[1])));
        const f2 k1 = add(mul_u(ax2, n[0]), neg(mul_u(ax0, n[2])));
        const f2 k2 = add(mul_u(ax0, n[1]), neg(mul_u(ax1, n[0])));
        dn[0] = add(dn[0], add(mul_u(n[0], cm1), mul_u(k0, sr)));
        dn[1] = add(dn[1], add(mul_u(n[1], cm1), mul_u(k1, sr)));
        dn[2] = add(dn[2], add(mul_u(n[2], cm1), mul_u(k2, sr)));
    }
    for (int k = 0; k < 3; ++k) o.dp[k] = dp[k];
    if (st.h >= 0x1p-10f) {
        const f2 stst = mul(st, st);
        const f2 nd = add(mul_u(n[0], dn[0]), mul_u(n[1], dn[1]));
        o.a = atan2_f2(add(mul_u(n[0], dn[1]), neg(mul_u(n[1], dn[0]))), add(stst, nd));
        // |v_xy| from v's components (st^2 + q cancels when v nears a pole);
        // its difference from st from q (which does not cancel)
        const f2 v0 = add(n[0], dn[0]), v1 = add(n[1], dn[1]);
        const f2 rxy = sqrt_f2(add(mul_u(v0, v0), mul_u(v1, v1)));
        const f2 q = add(add(nd, nd), add(mul_u(dn[0], dn[0]), mul_u(dn[1], dn[1])));
        const f2 delta = div_f2(q, add(rxy, st));
        o.b = atan2_f2(add(mul_u(delta, ct), neg(mul_u(dn[2], st))),
                       add(mul_u(rxy, st), mul_u(add(ct, dn[2]), ct)));
        o.direct = false;
    } else {
        const f2 v0 = add(n[0], dn[0]), v1 = add(n[1], dn[1]), v2 = add(n[2], dn[2]);
        o.a = atan2_f2(v1, v0);
        o.b = atan2_f2(v2, sqrt_f2(add(mul_u(v0, v0), mul_u(v1, v1))));
        o.direct = true;
    }
}

}  // namespace xf
}  // namespace ss
