// common.cuh -- device-side definitions shared by the timestep kernels.
//
// Data layout in HBM (one simulation per context):
//   particles   SoA doubles x[N], y[N], z[N], phi[N], theta[N]; uint32 key[N]
//               (spatial cell of the particle, index (ix*gy+iy)*gz+iz) and
//               uint32 id[N] (position in the caller's particle list).
//   counts      uint32 histogram [gx][gy][gz][gphi][gtheta] (two buffers:
//               the one this step's fields are built from, and the one the
//               particle update fills for the next step).
//   spectra     complex [9 stress (+3 polarisation)][ncell] forward buffer,
//               complex [9 grad u, 3 u (+9 grad B, 3 B)][ncell] inverse buffer.
//   table       one row of doubles per spatial cell with everything the
//               particle update gathers (TABLE_* offsets below).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace ss {

constexpr double kPi = 3.14159265358979323846;  // std::f64::consts::PI
constexpr double kTwoPi = 2.0 * kPi;             // src/consts.rs:8
constexpr double kPiHalf = kPi / 2.0;            // src/particle.rs:24

// ---- per-cell field table (doubles) ------------------------------------
constexpr int T_U = 0;      // Re u[3]                      (mod.rs:324)
constexpr int T_W01 = 3;    // Re W = (G - G^T)/2, W01 W02 W12 (mod.rs:302-306,325)
constexpr int T_W02 = 4;
constexpr int T_W12 = 5;
constexpr int T_E00 = 6;    // Re E = (G + G^T)/2, E00 E01 E02 E11 E12 E22 (mod.rs:307,326)
constexpr int T_E01 = 7;
constexpr int T_E02 = 8;
constexpr int T_E11 = 9;
constexpr int T_E12 = 10;
constexpr int T_E22 = 11;
constexpr int T_DIFF = 12;  // sqrt(2 dt (Dt + volume_exclusion*density)) (mod.rs:333-346)
constexpr int T_B = 13;     // Re B * magnetic_dipole_dipole [3]  (mod.rs:337-338)
constexpr int T_GB = 16;    // Re grad B [3][3]                   (mod.rs:339)
constexpr int T_DENS = 25;  // density, sum_a f * dtheta dphi (rows of stride 32 only)
constexpr int TABLE_STRIDE = 16;      // without the dipolar solver
constexpr int TABLE_STRIDE_MAG = 32;  // with it, or with the trilinear gather

// Langevin modifier bits, in the chain order of src/bin/simulation/mod.rs:348-363
enum : uint32_t {
    M_SELF_PROPULSION = 1u << 0,
    M_CONVECTION = 1u << 1,
    M_MDD_FORCE = 1u << 2,
    M_EXTERNAL_FIELD = 1u << 3,
    M_MDD_ROTATION = 1u << 4,
    M_JEFFREY_VORTICITY = 1u << 5,
    M_JEFFREY_STRAIN = 1u << 6,
    M_STEP = 1u << 7,
    M_TRANS_DIFFUSION = 1u << 8,
    M_ROT_DIFFUSION = 1u << 9,
    M_ALL = (1u << 10) - 1
};

// device error flags (host reads them after a synchronising call)
enum : uint32_t { ERR_BIN_RANGE = 1u, ERR_NONFINITE = 2u };

struct DevParams {
    int gx, gy, gz, gphi, gtheta;
    int ncell, nang;
    long long nbins;
    unsigned long long n;
    double bx, by, bz;
    double gw[5];    // GridWidth, src/mesh/grid_width.rs:23-31
    double igw[5];   // 1 / gw (only as a first guess for the bin index)
    double dt, Dt, Dr;
    double shape, drag, reorient, mdd, volex;
    double dist_den;   // gwx*gwy*gwz*gwphi*gwtheta*N (distribution/mod.rs:183)
    double volume;     // Lx*Ly*Lz (simulation/mod.rs:255-257)
    double measure;    // gwphi*gwtheta  (stress.rs:83, director.rs:237)
    double dthph;      // gwtheta*gwphi  (simulation/mod.rs:315)
    double sigma_rot;  // sqrt(2 Dr dt)  (simulation/mod.rs:267-270)
    double cos_half_pi, sin_half_pi;  // cos/sin of kPiHalf as evaluated on this device
    double shape_dt, reorient_dt;     // shape * dt, magnetic_reorientation * dt (canonical table)
    float dt2[2], reorient2[2], sigma2[2];  // dt, reorient_dt, sigma_rot as float pairs (hi, lo)
    float reorient_f2[2], shape2[2], drag2[2];  // magnetic_reorientation, shape, magnetic_drag as pairs
    int f32x2;         // the update's increments in two-float arithmetic (f32x2.cuh), nearest-cell gather
    float igwf[5];     // 1 / gw in FP32 (first estimate of the bin index)
    float bintol[5];   // half-width of the band around an integer where the FP32 estimate defers to FP64
    unsigned long long seed;
    int quasi2d;
    int bin_theta_half;  // the theta bin of pi/2 (every particle after a quasi2d step)
    int gather;        // 0 nearest cell, 1 trilinear, 2 trilinear with the z fraction from y
    int hdim[3];       // half-spectrum shape of the real-to-complex transforms: the last axis of size > 1 halved
    int nhalf;         // hdim[0] * hdim[1] * hdim[2]
    int cstride;       // component stride of the contraction's real fields: ncell rounded up to even, so
                       // every component starts 16-byte aligned (the real-to-complex transforms need it)
    uint32_t mask;     // Langevin modifiers that can change the state
};

// ---- reference arithmetic helpers -------------------------------------

// modulo, src/particle.rs:26-35.  fmod(x, m) is exact; for x in (-m, 2m) it
// equals x, x - m (exact by Sterbenz) or x (then + m), so the fast path gives
// the identical double without the fmod loop.
// Range tests on the bits.  For doubles with the sign bit clear the order of
// the bit patterns, as unsigned 64-bit integers, is the order of the values,
// so a test of a double against a positive bound is one unsigned compare on
// the integer pipe.  (A sign-magnitude key built with a select -- b < 0 ?
// -(b & mask) : b -- is recognised by the compiler as a double comparison
// and turned back into FP64 instructions: measured, 2 extra FP64 operations
// per range test.)
constexpr unsigned long long kSignBit = 0x8000000000000000ull;
__device__ __forceinline__ unsigned long long dbits(double d) { return (unsigned long long)__double_as_longlong(d); }

__device__ __forceinline__ double ref_modulo(double f, double m) {
    // m > 0 finite (box sizes, 2 pi); a NaN f fails both range tests and
    // goes through fmod as in the IEEE form of these compares
    const unsigned long long bf = dbits(f), bm = dbits(m);
    if (bf < bm || bf == kSignBit) return f;  // [+0, m) and -0.0: f itself, without an FP64 operation
    const bool neg = (bf & kSignBit) != 0;
    // (-m, 0): |f| < m; [m, 2m): bits below those of 2 m (the exponent of m plus one)
    if (neg ? (bf & ~kSignBit) < bm : bf < bm + (1ull << 52)) {
        // f + m or f - m; the sign of m is chosen on the integer pipe
        return f + __longlong_as_double((long long)(neg ? bm : (bm | kSignBit)));
    }
    double r = fmod(f, m);
    return (r < 0.0) ? r + fabs(m) : r;
}

// modulo for a position, which leaves the box rarely: the range test inline,
// the wrap in an out-of-line call.  The result is ref_modulo's, bit for bit.
static __device__ __noinline__ double modulo_wrap(double f, double m) { return ref_modulo(f, m); }
__device__ __forceinline__ double modulo_rare(double f, double m) {
    const unsigned long long bf = dbits(f);
    if (bf < dbits(m) || bf == kSignBit) return f;
    return modulo_wrap(f, m);
}

// ang_pbc, src/particle.rs:37-44
__device__ __forceinline__ void ref_ang_pbc(double &phi, double &theta) {
    double t = ref_modulo(theta, kTwoPi);
    // t > pi on the integer pipe (-0.0 and a NaN t compare false, as in FP64)
    const unsigned long long bt = dbits(t);
    if ((bt & kSignBit) == 0 && bt > dbits(kPi) && bt <= 0x7FF0000000000000ull) {
        phi = ref_modulo(phi + kPi, kTwoPi);
        theta = kTwoPi - t;
    } else {
        phi = ref_modulo(phi, kTwoPi);
        theta = t;
    }
}

// ---- FP64 <-> FP32 and floor in integer arithmetic ---------------------
// GB300 executes FP64 at 2 operations per clock per SM (FP32: 128), and a
// conversion, floor or compare occupies the FP64 pipe like an add; the
// integer pipes are many times wider.
//
// d2f_pos: the float nearest a double d (ties to even), the same as
// (float)d for d >= 2^-126; 0 for smaller or negative d.
__device__ __forceinline__ float d2f_pos(double d) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    const uint32_t e = (uint32_t)(b >> 52);  // biased exponent; >= 2048 when negative
    if (e < 1023u - 126u || e >= 2048u) return 0.0f;
    uint32_t f = ((e - 896u) << 23) | ((uint32_t)(b >> 29) & 0x7FFFFFu);
    const uint32_t rest = (uint32_t)b & 0x1FFFFFFFu;  // the 29 bits rounded off
    if (rest > 0x10000000u || (rest == 0x10000000u && (f & 1u))) f += 1u;
    return __uint_as_float(f);
}
// d2f: as (float)d for |d| >= 2^-126 or d == 0 (round to nearest is symmetric)
__device__ __forceinline__ float d2f(double d) {
    const long long b = __double_as_longlong(d);
    const float m = d2f_pos(__longlong_as_double(b & 0x7FFFFFFFFFFFFFFFll));
    return (b < 0) ? -m : m;
}
// f2d: the exact double of a float, all from its bits (zero, subnormals,
// inf and NaN included; a NaN keeps its payload bits)
__device__ __forceinline__ double f2d(float f) {
    const uint32_t u = __float_as_uint(f);
    const uint32_t e = (u >> 23) & 0xFFu, m = u & 0x7FFFFFu;
    unsigned long long body;
    if (e == 0xFFu) {
        body = (0x7FFull << 52) | ((unsigned long long)m << 29);
    } else if (e != 0u) {
        body = ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)m << 29);
    } else if (m == 0u) {
        body = 0ull;
    } else {  // subnormal m 2^-149 = 2^(p - 149) 1.f, p the highest set bit of m
        const int p = 31 - __clz(m);
        body = ((unsigned long long)(p + 874) << 52) | (((unsigned long long)m << (52 - p)) & 0xFFFFFFFFFFFFFull);
    }
    return __longlong_as_double((long long)(((unsigned long long)(u & 0x80000000u) << 32) | body));
}
// m 2^-52 rounded to the nearest float (ties to even) for 0 < m < 2^53,
// from m's bits (the value is a normal float, 2^-52 .. 2)
__device__ __forceinline__ float u52_to_float(unsigned long long m) {
    const int p = 63 - __clzll(m);  // 2^(p - 52) <= m 2^-52 < 2^(p - 51)
    unsigned long long q;
    if (p <= 23) {
        q = m << (23 - p);  // exact, the leading one at bit 23
    } else {
        const int sh = p - 23;
        q = m >> sh;
        const unsigned long long rest = m & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
        if (rest > half || (rest == half && (q & 1ull))) q += 1ull;  // a carry to 2^24 raises the exponent below
    }
    // exponent field p + 75, minus one for the leading one that q adds
    return __uint_as_float(((uint32_t)(p + 74) << 23) + (uint32_t)q);
}
// For 0 <= q < 2^31: fl = floor(q), and near = q lies within 2^-20 of an
// integer (fr = q - floor(q) < 2^-20 or fr > 1 - 2^-20), from q's bits.
// Returns false for other q (negative, -0.0, NaN, large).
__device__ __forceinline__ bool floor_near(double q, int &fl, bool &near) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(q);
    if (b >> 63) return false;
    const int e = (int)(b >> 52) - 1023;
    const unsigned long long m = b & 0xFFFFFFFFFFFFFull;
    if (e < 0) {  // [0, 1): floor 0; near 0 below 2^-20, near 1 above 1 - 2^-20
        fl = 0;
        near = e < -20 || (e == -1 && m > 0xFFFFFFFFFFFFFull - 0x1FFFFFFFFull);
        return true;
    }
    if (e >= 31) return false;
    const unsigned long long mant = m | (1ull << 52);
    const int shift = 52 - e;  // 22 .. 52
    fl = (int)(mant >> shift);
    const unsigned long long frac = mant & ((1ull << shift) - 1ull), tol = 1ull << (shift - 20);
    near = frac < tol || frac > (1ull << shift) - tol;
    return true;
}

// floor(v / w) as usize with the `== n -> n-1` clamp of
// Distribution::coord_to_grid (distribution/mod.rs:112-137) and
// get_cell_index (mesh/mod.rs:49-63).  v * (1/w) is within two ulps of the
// correctly rounded v / w; unless it lies within 2^-20 of an integer the two
// floors agree, otherwise the exact division decides.  Indices outside
// [0, n] (only reachable from non-finite or unwrapped input) are clamped and
// flagged.
__device__ __forceinline__ int ref_bin(double v, double w, double iw, int n, uint32_t &err) {
    double q = v * iw;
    {
        int fl;
        bool near;
        if (floor_near(q, fl, near) && !near) {  // the common case, without FP64 compares
            if (fl >= n) {
                if (fl > n) err |= ERR_BIN_RANGE;
                return n - 1;
            }
            return fl;
        }
    }
    double f = floor(q);
    double fr = q - f;
    if (fr < 0x1p-20 || fr > 1.0 - 0x1p-20) f = floor(v / w);
    int i;
    if (!(f >= 0.0)) {  // negative or NaN: Rust saturates to 0
        if (f != f || f < 0.0) err |= ERR_BIN_RANGE;
        i = 0;
    } else if (f >= (double)n) {
        if (f > (double)n) err |= ERR_BIN_RANGE;
        i = n - 1;
    } else {
        i = (int)f;
    }
    return i;
}

// ref_bin with a first estimate in FP32: q = float(v) * float(1/w) lies
// within 3 * 2^-24 * q (+ one ulp of 2^-126) of v / w.  When it is farther
// than tol = 8 * 2^-24 * (n + 1) from every integer (set on the host), the
// exact v / w and its FP64 rounding lie strictly between the same two
// integers, so floor(q) is the reference's index; otherwise (and for v
// outside [2^-126, 2^30), NaN included) ref_bin decides in FP64.
__device__ __forceinline__ int ref_bin_f(double v, double w, double iw, float iwf, float tol, int n,
                                         uint32_t &err) {
    const long long kv = __double_as_longlong(v);
    if (kv >= 0x3810000000000000ll && kv < 0x41D0000000000000ll) {  // [2^-126, 2^30)
        const float q = d2f_pos(v) * iwf;
        const float fl = floorf(q), fr = q - fl;
        if (fr > tol && fr < 1.0f - tol) {
            const int i = (int)fl;
            if (i >= n) {
                if (i > n) err |= ERR_BIN_RANGE;
                return n - 1;
            }
            return i;
        }
    }
    return ref_bin(v, w, iw, n, err);
}

// ---- Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) -----------------
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
    constexpr uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    constexpr uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0 = __umulhi(M0, c.x), lo0 = M0 * c.x;
        uint32_t hi1 = __umulhi(M1, c.z), lo1 = M1 * c.z;
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
        k.x += W0;
        k.y += W1;
    }
    return c;
}

// A double in [1, 2) whose 52 mantissa bits come from two 32-bit words,
// assembled with integer operations (no FP64 conversion).  x - 1 is a uniform
// in [0, 1) and 2 - x one in (0, 1], both exact.
__device__ __forceinline__ double u12(uint32_t hi, uint32_t lo) {
    return __hiloint2double((int)(0x3FF00000u | (hi >> 12)), (int)((hi << 20) | (lo >> 12)));
}

// -2 ln(1 - U) in FP32 with full relative precision over all of (0, 1],
// from x = 1 + U in [1, 2) (52 random bits, U = m 2^-52 with m the mantissa
// of x): log1p takes -U below U = 1/2 (the radius near 0), log takes
// 1 - U = (2^52 - m) 2^-52 above it (the tail, down to 1 - U = 2^-52).  Both
// arguments are the float nearest the exact value, formed from m's bits
// (the same floats as rounding the exact FP64 differences 1 - x and 2 - x).
__device__ __forceinline__ float neg2log1m(double x) {
    const unsigned long long m = (unsigned long long)__double_as_longlong(x) & 0xFFFFFFFFFFFFFull;
    const float l = (m >> 51) == 0ull ? log1pf(m ? -u52_to_float(m) : 0.0f)
                                      : logf(u52_to_float((1ull << 52) - m));
    return -2.0f * l;
}

// Noise of particle `id` at step `t`: the RandomVector of
// src/bin/simulation/mod.rs:272-286 (x, y, z ~ N(0,1), axis_angle = 2 pi U,
// rotate_angle = sigma sqrt(-2 ln(1-U))), drawn from Philox with counter
// (id, t_lo, t_hi, draw) and key = seed.  Normals by Box-Muller.
//
// The transcendentals of the noise run in FP32 (the FP64 pipe is the scarce
// unit of the update); every value handed to the FP64 step is an exact double
// of that FP32 result, and ss_noise returns the same doubles, so the FP64
// oracle fed ss_noise sees exactly what the update used.  Radii take 52-bit
// uniforms through neg2log1m (tails to 8.5 sigma); angles take 24-bit
// uniforms.  The axis angle is returned as its sine and cosine: the sine is
// the FP32 sine (an exact double), the cosine sqrt(1 - sine^2) in FP64 with
// the sign of the FP32 cosine, a unit pair to FP64 rounding, so that
// sincos(atan2(sa, ca)) reproduces (ca, sa) to FP64 rounding.  The
// canonical quasi-2-D chain reads only the sine, which then costs no FP64
// operation.
// The FP32 draws of the first two Philox blocks: the normals xi0, xi1, the
// sine and cosine of the axis angle and the Rayleigh radius of the rotation
// angle before sigma (philox_noise turns them into exact doubles; the
// two-float update uses them as they are).
struct NoiseF {
    float xi0, xi1, sa, ca, rad;
};
__device__ __forceinline__ NoiseF philox_noise_f(unsigned long long seed, uint32_t id, unsigned long long t) {
    const uint2 key = make_uint2((uint32_t)seed, (uint32_t)(seed >> 32));
    const uint32_t tl = (uint32_t)t, th = (uint32_t)(t >> 32);
    const uint4 r0 = philox4x32_10(make_uint4(id, tl, th, 0u), key);
    const uint4 r1 = philox4x32_10(make_uint4(id, tl, th, 1u), key);
    NoiseF f;
    const float rad = sqrtf(neg2log1m(u12(r0.x, r0.y)));
    float s, c;
    sincospif(2.0f * (float)(r0.z >> 8) * 0x1p-24f, &s, &c);
    f.xi0 = rad * c;
    f.xi1 = rad * s;
    sincospif(2.0f * (float)(r1.x >> 8) * 0x1p-24f, &f.sa, &f.ca);
    f.rad = sqrtf(neg2log1m(u12(r1.z, r1.w)));
    return f;
}

// The third normal (the z component of the translational noise, 3-D steps)
// as its FP32 value, from the third Philox block.
__device__ __forceinline__ float philox_xi2_f(unsigned long long seed, uint32_t id, unsigned long long t) {
    const uint2 key = make_uint2((uint32_t)seed, (uint32_t)(seed >> 32));
    const uint4 r2 = philox4x32_10(make_uint4(id, (uint32_t)t, (uint32_t)(t >> 32), 2u), key);
    const float rad2 = sqrtf(neg2log1m(u12(r2.x, r2.y)));
    return rad2 * cospif(2.0f * (float)(r2.z >> 8) * 0x1p-24f);
}

template <bool Q2D, bool WANT_ALPHA = false>
__device__ __forceinline__ void philox_noise(unsigned long long seed, uint32_t id, unsigned long long t,
                                             double sigma, double xi[3], double &ca, double &sa,
                                             double &rot, double *alpha = nullptr) {
    const NoiseF f = philox_noise_f(seed, id, t);
    xi[0] = f2d(f.xi0);
    xi[1] = f2d(f.xi1);
    xi[2] = Q2D ? 0.0 : f2d(philox_xi2_f(seed, id, t));  // quasi2d: z is overwritten, never read
    sa = f2d(f.sa);
    ca = sqrt(fma(-sa, sa, 1.0));  // |sa| <= 1: the argument is >= 0
    ca = __longlong_as_double(__double_as_longlong(ca) | ((long long)(__float_as_uint(f.ca) >> 31) << 63));
    rot = sigma * f2d(f.rad);
    if (WANT_ALPHA) {
        double a = atan2(sa, ca);
        *alpha = a < 0.0 ? a + kTwoPi : a;
    }
}

// ---- sin, cos and atan2 from a table of j / 128 -------------------------
// kTrig[j] = (cos a_j, sin a_j) and kTrigCm1[j] = cos a_j - 1 at a_j = j / 128,
// correctly rounded (gen_trig_table.py).  An angle a_j + b with |b| <= 2^-8
// needs only short Taylor polynomials in b and the addition theorem: about
// 12 FP64 operations for sin and cos and 16 for atan2, where the general
// routines spend an argument reduction and long polynomials on the FP64
// pipe (the bound of the update).  sin and cos are within 1.7e-16 of the
// correctly rounded values (an ulp of 1; relative to a value near a zero
// of sin or cos that is more than an ulp), atan2 within 2 ulp.
#include "trig_table.inc"

// j = round(128 a) for +0 <= a < 6.3, from a's bits on the integer pipe;
// -1 for other a (negative, -0.0, larger, NaN)
__device__ __forceinline__ int trig_round(double a) {
    const long long bits = __double_as_longlong(a);
    if (bits < 0 || bits >= kTrigMaxKey) return -1;
    const int e = (int)(bits >> 52) - 1023;
    if (e < -9) return 0;  // a < 2^-9: 128 a < 1/4
    const unsigned long long mant = (unsigned long long)(bits & 0xFFFFFFFFFFFFFll) | (1ull << 52);
    const int shift = 45 - e;  // 128 a = mant 2^-shift, shift in 43 .. 54
    return (int)((mant + (1ull << (shift - 1))) >> shift);
}

// a_j = j / 128 as a double, from j's bits (0 <= j < 2^20)
__device__ __forceinline__ double trig_angle(int j) {
    if (j == 0) return 0.0;
    const int hb = 31 - __clz(j);
    const unsigned long long b = ((unsigned long long)(1023 + hb - 7) << 52) |
                                 (((unsigned long long)j << (52 - hb)) & 0xFFFFFFFFFFFFFull);
    return __longlong_as_double((long long)b);
}

// sin b and cos b - 1 for |b| <= 2^-8 (+ a few FP32 ulps): Taylor to b^5 and
// b^4.  The first omitted terms are below 4e-18 relative (sin) and 1.2e-17
// absolute (cos b - 1, relative 7e-13): every caller adds cos b - 1 times a
// factor of at most 1 to a value of order 1, where 1.2e-17 is a tenth of an
// ulp.
__device__ __forceinline__ void trig_small(double b, double &sb, double &cb) {
    const double z = b * b;
    sb = fma(b * z, fma(z, 1.0 / 120.0, -1.0 / 6.0), b);
    cb = z * fma(z, 1.0 / 24.0, -0.5);
}

// sin a and cos a (sincos for a outside [0, 6.3))
__device__ __forceinline__ void tab_sincos(double a, double &s, double &c) {
    const int j = trig_round(a);
    if (j < 0) {
        sincos(a, &s, &c);
        return;
    }
    const double b = a - trig_angle(j);  // exact: a_j is a multiple of ulp(a), |b| <= min(a, 2^-8)
    const double2 t = __ldg(&kTrig[j]);
    double sb, cb;
    trig_small(b, sb, cb);
    s = fma(t.x, sb, fma(t.y, cb, t.y));
    c = fma(-t.y, sb, fma(t.x, cb, t.x));
}

// sin r and cos r - 1, the latter without the cancellation of cos r - 1
// (from cos a_j - 1; within about an ulp of its own size)
__device__ __forceinline__ void sin_cosm1(double r, double &s, double &cm1) {
    const int j = trig_round(r);
    if (j < 0) {
        double c;
        sincos(r, &s, &c);
        cm1 = c - 1.0;
        return;
    }
    const double b = r - trig_angle(j);
    const double2 t = __ldg(&kTrig[j]);
    const double tm = __ldg(&kTrigCm1[j]);
    double sb, cb;
    trig_small(b, sb, cb);
    s = fma(t.x, sb, fma(t.y, cb, t.y));
    cm1 = fma(t.x, cb, fma(-t.y, sb, tm));  // (cos a_j - 1) + cos a_j (cos b - 1) - sin a_j sin b
}

// atan2(y, x).  An FP32 estimate of the angle of (x, |y|) picks a_j; the
// vector rotated by -a_j has the small angle eps = atan(e / d), |eps| <=
// 2^-8 + 1e-6, from an FP64 quotient (FP32 reciprocal, two Newton steps)
// and the series eps - eps^3/3 + eps^5/5 - eps^7/7 (omitted terms below
// 1e-20 relative); the sign of y is applied last (atan2 is odd in y).
// Inputs whose rotated length d is not a positive number in [2^-60, 2^61),
// or whose |e| is not below d 2^-8 (zero, tiny, huge or non-finite vectors,
// for which the FP32 estimate fails) go through atan2.
__device__ __forceinline__ double tab_atan2(double y, double x) {
    const float af = atan2f(fabsf(d2f(y)), d2f(x));  // [0, pi] to ~1e-7 (NaN -> j = 0)
    const int j = __float2int_rn(af * 128.0f);       // 0 .. 402
    const double2 t = __ldg(&kTrig[j]);
    const double ay = fabs(y);
    const double d = fma(ay, t.y, x * t.x);   // along a_j
    const double e = fma(-x, t.y, ay * t.x);  // across it
    const long long db = __double_as_longlong(d);
    const int ed = (int)(db >> 52), ee = (int)((__double_as_longlong(e) >> 52) & 0x7FF);
    if (db < 0x3C30000000000000ll || db >= 0x43C0000000000000ll || ee > ed - 8) return atan2(y, x);
    const double r0 = f2d(__frcp_rn(d2f_pos(d)));
    const double r = fma(r0, fma(-d, r0, 1.0), r0);  // 1 / d to ~2^-46
    const double q = e * r;
    const double eps = fma(r, fma(-d, q, e), q);     // e / d to about an ulp
    const double z = eps * eps;
    const double at = fma(eps * z, fma(z, fma(z, -1.0 / 7.0, 1.0 / 5.0), -1.0 / 3.0), eps);
    const double ang = trig_angle(j) + at;
    return __longlong_as_double(__double_as_longlong(ang) ^ (__double_as_longlong(y) & (long long)0x8000000000000000ull));
}

// ---- the Langevin chain ------------------------------------------------
// Field access for the chain.  TableFields reads one row of the per-cell
// table; MatrixFields carries full 3x3 matrices (used by ss_langevin).
struct TableFields {
    const double *r;
    __device__ double flow(int k) const { return r[T_U + k]; }
    __device__ double diff() const { return r[T_DIFF]; }
    __device__ double b(int k) const { return r[T_B + k]; }
    // Array2.dot(Array1) row a, then * (-1): ((0 + W[a][0]n0) + W[a][1]n1) + W[a][2]n2
    // with W[a][a] == 0 exactly and W[b][a] == -W[a][b] exactly.
    __device__ void vort_dot(const double n[3], double f[3]) const {
        double w01 = r[T_W01], w02 = r[T_W02], w12 = r[T_W12];
        f[0] = w01 * n[1] + w02 * n[2];
        f[1] = (-w01) * n[0] + w12 * n[2];
        f[2] = (-w02) * n[0] + (-w12) * n[1];
    }
    __device__ void strain_dot(const double n[3], double f[3]) const {
        double e00 = r[T_E00], e01 = r[T_E01], e02 = r[T_E02], e11 = r[T_E11], e12 = r[T_E12],
               e22 = r[T_E22];
        f[0] = (e00 * n[0] + e01 * n[1]) + e02 * n[2];
        f[1] = (e01 * n[0] + e11 * n[1]) + e12 * n[2];
        f[2] = (e02 * n[0] + e12 * n[1]) + e22 * n[2];
    }
    __device__ void gradb_dot(const double n[3], double f[3]) const {
        const double *g = r + T_GB;
#pragma unroll
        for (int a = 0; a < 3; ++a) f[a] = (g[3 * a] * n[0] + g[3 * a + 1] * n[1]) + g[3 * a + 2] * n[2];
    }
};

struct MatrixFields {
    const double *flow_, *gradb_, *b_, *vort_, *strain_;
    double diff_;
    __device__ double flow(int k) const { return flow_[k]; }
    __device__ double diff() const { return diff_; }
    __device__ double b(int k) const { return b_[k]; }
    static __device__ void rowdot(const double *m, const double n[3], double f[3]) {
#pragma unroll
        for (int a = 0; a < 3; ++a) f[a] = (m[3 * a] * n[0] + m[3 * a + 1] * n[1]) + m[3 * a + 2] * n[2];
    }
    __device__ void vort_dot(const double n[3], double f[3]) const { rowdot(vort_, n, f); }
    __device__ void strain_dot(const double n[3], double f[3]) const { rowdot(strain_, n, f); }
    __device__ void gradb_dot(const double n[3], double f[3]) const { rowdot(gradb_, n, f); }
};

// Trilinear gather (src/mesh/interpolate.rs:11-119): the fields at the
// particle position from the eight surrounding cell centres, periodic.
// q = position / grid width; fraction fmod(q + 0.5, 1) (:19-23, with the
// reference's y in place of z when zbug), lower corner floor(q - 0.5)
// (:68-78), lerp a (1 - t) + b t (lerp 0.2.0) along x, then y, then z
// (:104-119).  The interpolated row holds u, W, E, B mdd, grad B and the
// density; the diffusion length is formed from the interpolated density.
template <bool MAG>
__device__ __forceinline__ void trilinear_row(const double *__restrict__ table, const DevParams &P, double x,
                                              double y, double z, double *row) {
    double qx = x / P.gw[0], qy = y / P.gw[1], qz = z / P.gw[2];
    double ax = qx + 0.5, ay = qy + 0.5, az = (P.gather == 2 ? y / P.gw[2] : qz) + 0.5;
    double t[3] = {ax - floor(ax), ay - floor(ay), az - floor(az)};  // fmod(., 1) for a >= 0, exact
    int n[3] = {P.gx, P.gy, P.gz};
    double lo[3] = {floor(qx - 0.5), floor(qy - 0.5), floor(qz - 0.5)};
    int c[3][2];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        int i = (int)lo[k];
        c[k][0] = (i + n[k]) % n[k];
        c[k][1] = (i + 1 + n[k]) % n[k];
    }
    const double *r[2][2][2];
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b)
#pragma unroll
            for (int d = 0; d < 2; ++d)
                r[a][b][d] = table + (long long)((c[0][a] * P.gy + c[1][b]) * P.gz + c[2][d]) * TABLE_STRIDE_MAG;
    const double sx = 1.0 - t[0], sy = 1.0 - t[1], sz = 1.0 - t[2];
    auto lerp3 = [&](int j) {
        double c00 = r[0][0][0][j] * sx + r[1][0][0][j] * t[0];
        double c01 = r[0][0][1][j] * sx + r[1][0][1][j] * t[0];
        double c10 = r[0][1][0][j] * sx + r[1][1][0][j] * t[0];
        double c11 = r[0][1][1][j] * sx + r[1][1][1][j] * t[0];
        double c0 = c00 * sy + c10 * t[1];
        double c1 = c01 * sy + c11 * t[1];
        return c0 * sz + c1 * t[2];
    };
#pragma unroll
    for (int j = 0; j < 12; ++j) row[j] = lerp3(j);
    if (MAG) {
#pragma unroll
        for (int j = T_B; j < T_GB + 9; ++j) row[j] = lerp3(j);
    }
    double dens = lerp3(T_DENS);
    row[T_DIFF] = sqrt(2.0 * P.dt * (P.Dt + P.volex * dens));
}

// One particle through LangevinBuilder::new -> modifiers -> step -> noise ->
// finalize (src/integrators/langevin_builder/mod.rs:25-125,
// modifiers.rs:39-231, particle.rs:106-121,219-222), then the quasi2d override
// (simulation/mod.rs:365-368).  Terms whose coefficient is exactly zero are
// masked off by the caller: they add an exact +-0 in the reference.
//   cth/sth: cos/sin of theta when the caller knows them (quasi2d), else pass
//   have_theta = false.  (ca, sa): cos/sin of the rotation axis angle.
template <bool Q2D, class F>
__device__ __forceinline__ void langevin(double &x, double &y, double &z, double &phi, double &theta,
                                         const F &fld, const double xi[3], double ca, double sa, double rot,
                                         uint32_t mask, double dt, double reorient, double shape, double drag,
                                         double bx, double by, double bz, bool have_theta, double cth,
                                         double sth) {
    double sp, cp, ct, st;
    tab_sincos(phi, sp, cp);
    if (have_theta) {
        ct = cth;
        st = sth;
    } else {
        tab_sincos(theta, st, ct);
    }
    // CosSinOrientation::to_orientation_vector, particle.rs:165-172
    // (with sin(theta) == 1 exactly, the products are cp and sp exactly)
    double n[3];
    if (have_theta && __double_as_longlong(st) == __double_as_longlong(1.0)) {
        n[0] = cp;
        n[1] = sp;
    } else {
        n[0] = st * cp;
        n[1] = st * sp;
    }
    n[2] = ct;
    double dp[3] = {0.0, 0.0, 0.0}, dn[3] = {0.0, 0.0, 0.0};

    if (mask & M_SELF_PROPULSION) {  // modifiers.rs:39-46
        dp[0] = n[0]; dp[1] = n[1]; dp[2] = n[2];
    }
    if (mask & M_CONVECTION) {  // modifiers.rs:49-56
#pragma unroll
        for (int k = 0; k < 3; ++k) dp[k] = dp[k] + fld.flow(k);
    }
    if (mask & M_MDD_FORCE) {  // modifiers.rs:59-70
        double f[3];
        fld.gradb_dot(n, f);
#pragma unroll
        for (int k = 0; k < 3; ++k) dp[k] = dp[k] + f[k] * drag;
    }
    if (mask & M_EXTERNAL_FIELD) {  // modifiers.rs:103-119 (field along y)
        double b[3] = {0.0, reorient, 0.0};
        double d = (n[0] * b[0] + n[1] * b[1]) + n[2] * b[2];
#pragma unroll
        for (int k = 0; k < 3; ++k) dn[k] = dn[k] + (b[k] - n[k] * d);
    }
    if (mask & M_MDD_ROTATION) {  // modifiers.rs:172-187
        double b[3] = {fld.b(0), fld.b(1), fld.b(2)};
        double d = (n[0] * b[0] + n[1] * b[1]) + n[2] * b[2];
#pragma unroll
        for (int k = 0; k < 3; ++k) dn[k] = dn[k] + (b[k] - n[k] * d);
    }
    if (mask & M_JEFFREY_VORTICITY) {  // modifiers.rs:123-143
        double f[3];
        fld.vort_dot(n, f);
#pragma unroll
        for (int k = 0; k < 3; ++k) dn[k] = dn[k] + (-f[k]);
    }
    if (mask & M_JEFFREY_STRAIN) {  // modifiers.rs:147-170
        double f[3];
        fld.strain_dot(n, f);
#pragma unroll
        for (int k = 0; k < 3; ++k) f[k] = f[k] * shape;
        double fn = (f[0] * n[0] + f[1] * n[1]) + f[2] * n[2];
#pragma unroll
        for (int k = 0; k < 3; ++k) dn[k] = dn[k] + (f[k] - n[k] * fn);
    }
    if (mask & M_STEP) {  // mod.rs:114-119
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            dp[k] = dp[k] * dt;
            dn[k] = dn[k] * dt;
        }
    }
    if (mask & M_TRANS_DIFFUSION) {  // modifiers.rs:86-99
        double diff = fld.diff();
#pragma unroll
        for (int k = 0; k < 3; ++k) dp[k] = dp[k] + xi[k] * diff;
    }
    if (mask & M_ROT_DIFFUSION) {  // modifiers.rs:199-231
        // Rotation axis k perpendicular to n (modifiers.rs:205-215).  The
        // reference rotates with the quaternion q n q* of
        // quaternion::axis_angle(k, rot) (quaternion 0.3.1); for a unit k
        // perpendicular to n that rotation is n cos(rot) + (k x n) sin(rot)
        // (Rodrigues), which needs one sincos and a cross product instead of
        // two quaternion products.  The delta R n - n is formed as
        // n (cos - 1) + (k x n) sin, without the cancellation of R n - n.
        double ax0 = (cp * ct) * sa - ca * sp;
        double ax1 = ca * cp + (ct * sa) * sp;
        double ax2 = (-sa) * st;
        double sr, cm1;
        sin_cosm1(rot, sr, cm1);
        double k0 = ax1 * n[2] - ax2 * n[1];
        double k1 = ax2 * n[0] - ax0 * n[2];
        double k2 = ax0 * n[1] - ax1 * n[0];
        dn[0] = dn[0] + (n[0] * cm1 + k0 * sr);
        dn[1] = dn[1] + (n[1] * cm1 + k1 * sr);
        dn[2] = dn[2] + (n[2] * cm1 + k2 * sr);
    }
    // finalize: Particle::from(old + delta) then pbc (mod.rs:121-125)
    double px = x + dp[0], py = y + dp[1], pz = z + dp[2];
    double v0 = n[0] + dn[0], v1 = n[1] + dn[1], v2 = n[2] + dn[2];
    double nphi = tab_atan2(v1, v0);  // Orientation::from_vector, particle.rs:106-121
    x = modulo_rare(px, bx);
    y = modulo_rare(py, by);
    if (Q2D) {
        // theta = pi/2 - atan2(v2, rxy) lies in [0, pi] (rxy >= 0), so
        // ang_pbc only wraps phi; z and theta are overwritten (mod.rs:365-368).
        phi = ref_modulo(nphi, kTwoPi);
        z = 0.0;
        theta = kPiHalf;
    } else {
        double rxy = sqrt(v0 * v0 + v1 * v1);
        double nth = kPiHalf - tab_atan2(v2, rxy);
        z = modulo_rare(pz, bz);
        ref_ang_pbc(nphi, nth);
        phi = nphi;
        theta = nth;
    }
}

// Row of the canonical table (k_table, for quasi2d steps without the
// dipolar solver): the fields the canonical chain reads, pre-multiplied by
// dt: u0 dt, u1 dt, W01 dt, shape dt E00, shape dt E01, shape dt E11, the
// diffusion length, 0.
constexpr int CT_U0 = 0, CT_U1 = 1, CT_W01 = 2, CT_E00 = 3, CT_E01 = 4, CT_E11 = 5, CT_DIFF = 6;
constexpr int CTAB_STRIDE = 8;

// The chain of `langevin` for a quasi-2-D particle in the canonical state
// (theta = pi/2 and z = 0, which every particle holds after a quasi2d step)
// and no magnetic modifiers: n = (cos phi, sin phi, cos(pi/2)) with
// cos(pi/2) (6.1e-17 in FP64) taken as 0 and sin(pi/2) == 1 exactly, so the
// products with n_z and every z component drop out.  The step's factor dt is
// applied to the fields once per cell (the canonical table) instead of to
// every particle's sums.  In the plane every deterministic orientation
// term is a multiple of n_perp = (-sin phi, cos phi): the external field
// (0, r, 0) gives (r cos phi) n_perp, the vorticity W01 n_perp, the strain
// (n_perp . f) n_perp, and the rotational diffusion turns n into
// n cos rot - sa sin rot n_perp.  So v = n + dn = C n + G n_perp with
// C = cos rot and G the sum of those coefficients, and the new angle
// atan2(v) is phi + atan2(G, C), formed without v.  Each regrouped or
// dropped product is below half an ulp of the sum it joins, so the results
// can differ from the full chain's in the last bits, like the rounding of
// sin / cos / atan2.  z and theta are not produced (the quasi2d step
// overwrites them with 0 and pi/2, which the canonical state already holds).
__device__ __forceinline__ void langevin_canon(double &x, double &y, double &phi, const double *__restrict__ ct,
                                               const double xi[3], double sa, double rot, uint32_t mask, double dt,
                                               double reorient_dt, double bx, double by) {
    double sp, cp;
    tab_sincos(phi, sp, cp);
    const double2 c01 = __ldg(reinterpret_cast<const double2 *>(ct));       // u0 dt, u1 dt
    const double2 c23 = __ldg(reinterpret_cast<const double2 *>(ct) + 1);   // W01 dt, s E00
    const double2 c45 = __ldg(reinterpret_cast<const double2 *>(ct) + 2);   // s E01, s E11
    const double2 c67 = __ldg(reinterpret_cast<const double2 *>(ct) + 3);   // diffusion length, 0
    double dp0, dp1;
    if ((mask & M_SELF_PROPULSION) && (mask & M_CONVECTION)) {
        dp0 = fma(cp, dt, c01.x);
        dp1 = fma(sp, dt, c01.y);
    } else if (mask & M_SELF_PROPULSION) {
        dp0 = cp * dt;
        dp1 = sp * dt;
    } else if (mask & M_CONVECTION) {
        dp0 = c01.x;
        dp1 = c01.y;
    } else {
        dp0 = 0.0;
        dp1 = 0.0;
    }
    if (mask & M_TRANS_DIFFUSION) {
        dp0 = fma(xi[0], c67.x, dp0);
        dp1 = fma(xi[1], c67.x, dp1);
    }
    // the coefficient of n_perp, term by term in the reference's order
    double G = 0.0;
    if (mask & M_EXTERNAL_FIELD) G = reorient_dt * cp;  // b - n (n . b), b = (0, r dt, 0)
    if (mask & M_JEFFREY_VORTICITY) G = (mask & M_EXTERNAL_FIELD) ? G + c23.x : c23.x;  // -(W n) dt
    if (mask & M_JEFFREY_STRAIN) {  // f - n (f . n), f = shape dt E n
        const double f0 = fma(c23.y, cp, c45.x * sp), f1 = fma(c45.x, cp, c45.y * sp);
        G = G + fma(cp, f1, -(sp * f0));
    }
    double C = 1.0;
    if (mask & M_ROT_DIFFUSION) {  // n cos rot + (k x n) sin rot, k x n = -sa n_perp
        double sr;
        tab_sincos(rot, sr, C);
        G = fma(-sa, sr, G);
    }
    const double px = x + dp0, py = y + dp1;
    x = modulo_rare(px, bx);
    y = modulo_rare(py, by);
    phi = ref_modulo(phi + tab_atan2(G, C), kTwoPi);
}

}  // namespace ss
