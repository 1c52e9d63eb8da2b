// mixed_device.cuh -- device functions of the FP32 mixed-precision step,
// shared by the single-simulation kernels (mixed.cu) and the batched
// ensemble (ensemble.cu).
#pragma once

#include "mixed.cuh"

namespace ss {

__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ float kval_f(int i, int n, float step) {
    int b = (n % 2 == 0) ? n / 2 : n / 2 + 1;
    return (float)(i < b ? i : i - n) * step;
}

// floor(v / w) in FP32 with the `== n -> n - 1` clamp of coord_to_grid
__device__ __forceinline__ int bin_f(float v, float iw, int n) {
    float f = floorf(v * iw);
    int i = (int)f;
    i = i < 0 ? 0 : i;
    return i >= n ? n - 1 : i;
}

__device__ __forceinline__ float modulo_f(float f, float m) {
    float r = fmodf(f, m);
    return r < 0.0f ? r + fabsf(m) : r;
}

// (d2f_pos and f2d, the integer-pipe conversions, are in common.cuh)

__device__ __forceinline__ void bin_mixed(const MixedParams &M, double x, double y, double z, float phi, float theta,
                                          uint32_t &cell, unsigned long long &bin) {
    int ix = bin_f(d2f_pos(x), M.igwf[0], M.gx);
    int iy = bin_f(d2f_pos(y), M.igwf[1], M.gy);
    int iz = bin_f(d2f_pos(z), M.igwf[2], M.gz);
    int ip = bin_f(phi, M.igwf[3], M.gphi);
    int it = bin_f(theta, M.igwf[4], M.gtheta);
    cell = (uint32_t)((ix * M.gy + iy) * M.gz + iz);
    bin = (unsigned long long)cell * (unsigned long long)M.nang + (unsigned long long)(ip * M.gtheta + it);
}

// ---- 64-bit fixed-point positions (SS_FLAG_FIXED64) ----------------------
// A coordinate x in [0, L) is stored as X = x / L * 2^64 in a u64 (the same
// 8 bytes as the double it replaces).  Adding a step is a 64-bit integer add;
// leaving the box on either side wraps modulo 2^64, which is the periodic
// boundary.  The cell is floor(X * n / 2^64), the high word of a 64-bit
// product, exact.  The resolution, L / 2^64, is 2^11 times finer than FP64
// near x = L.
__device__ __forceinline__ unsigned long long to_fixed(double x, double L) {
    double q = x / L;  // in [0, 1)
    unsigned long long X = (unsigned long long)(q * 0x1p64 >= 0x1p64 ? 0x1p64 - 2048.0 : q * 0x1p64);
    return X;
}
__device__ __forceinline__ double from_fixed(unsigned long long X, double unit) { return (double)X * unit; }
// FP32 step -> signed fixed-point increment, in two 32-bit halves (no FP64)
__device__ __forceinline__ unsigned long long step_fixed(float dx, float s32) {
    float s = dx * s32;            // the step in units of 2^-32 L
    s = fminf(fmaxf(s, -0x1p31f + 256.f), 0x1p31f - 256.f);  // |step| < L / 2
    float hf = floorf(s);
    int hi = (int)hf;
    uint32_t lo = (uint32_t)((s - hf) * 0x1p32f);
    return ((unsigned long long)(long long)hi << 32) + (unsigned long long)lo;
}
__device__ __forceinline__ int cell_fixed(unsigned long long X, int n) {
    return (int)__umul64hi(X, (unsigned long long)n);
}

// ---- the particle update ----------------------------------------------
__device__ __forceinline__ float u24(uint32_t r) { return (float)(r >> 8) * 0x1p-24f; }

template <bool Q2D>
__device__ __forceinline__ void philox_noise_f(unsigned long long seed, uint32_t id, unsigned long long t,
                                               float sigma, float xi[3], float &ca, float &sa, float &rot) {
    uint2 key = make_uint2((uint32_t)seed, (uint32_t)(seed >> 32));
    uint32_t tl = (uint32_t)t, th = (uint32_t)(t >> 32);
    uint4 r0 = philox4x32_10(make_uint4(id, tl, th, 0u), key);
    // the noise needs only statistical accuracy: the hardware approximations
    // (__logf: relative error ~2^-21 on (2^-24, 1]; __sincosf: absolute
    // error ~2^-21 on [-pi, pi], where the angles are drawn)
    constexpr float kTwoPiF = 6.28318530717958647692f;
    float rad = sqrtf(-2.0f * __logf(1.0f - u24(r0.x)));
    float s, c;
    __sincosf(kTwoPiF * (u24(r0.y) - 0.5f), &s, &c);
    xi[0] = rad * c;
    xi[1] = rad * s;
    __sincosf(kTwoPiF * (u24(r0.z) - 0.5f), &sa, &ca);
    rot = sigma * sqrtf(-2.0f * __logf(1.0f - u24(r0.w)));
    if (Q2D) {
        xi[2] = 0.f;
    } else {
        uint4 r1 = philox4x32_10(make_uint4(id, tl, th, 1u), key);
        xi[2] = sqrtf(-2.0f * __logf(1.0f - u24(r1.x))) * __cosf(kTwoPiF * (u24(r1.y) - 0.5f));
    }
}

// One row of the FP32 field table: the first 16 floats (u, W, E, the
// diffusion length, mdd B) are read with four 16-byte loads when the row is
// opened; the dipolar gradient (floats 16-24 of a 32-float row) on demand.
struct TableFieldsF {
    const float *r;
    float v[16];
    __device__ __forceinline__ explicit TableFieldsF(const float *row) : r(row) {
        const float4 *q = reinterpret_cast<const float4 *>(row);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float4 t = __ldg(q + k);
            v[4 * k] = t.x;
            v[4 * k + 1] = t.y;
            v[4 * k + 2] = t.z;
            v[4 * k + 3] = t.w;
        }
    }
    __device__ float flow(int k) const { return v[T_U + k]; }
    __device__ float diff() const { return v[T_DIFF]; }
    __device__ float b(int k) const { return v[T_B + k]; }
    __device__ void vort_dot(const float n[3], float f[3]) const {
        float w01 = v[T_W01], w02 = v[T_W02], w12 = v[T_W12];
        f[0] = w01 * n[1] + w02 * n[2];
        f[1] = -w01 * n[0] + w12 * n[2];
        f[2] = -w02 * n[0] - w12 * n[1];
    }
    __device__ void strain_dot(const float n[3], float f[3]) const {
        float e00 = v[T_E00], e01 = v[T_E01], e02 = v[T_E02], e11 = v[T_E11], e12 = v[T_E12], e22 = v[T_E22];
        f[0] = e00 * n[0] + e01 * n[1] + e02 * n[2];
        f[1] = e01 * n[0] + e11 * n[1] + e12 * n[2];
        f[2] = e02 * n[0] + e12 * n[1] + e22 * n[2];
    }
    __device__ void gradb_dot(const float n[3], float f[3]) const {
        const float *g = r + T_GB;
#pragma unroll
        for (int a = 0; a < 3; ++a) f[a] = g[3 * a] * n[0] + g[3 * a + 1] * n[1] + g[3 * a + 2] * n[2];
    }
};

// The Langevin chain of do_timestep in FP32, positions accumulated in FP64.
template <bool Q2D>
__device__ __forceinline__ void langevin_mixed(float &phi, float &theta, float step[3], const TableFieldsF &fld,
                                               const float xi[3], float ca, float sa, float rot,
                                               const MixedParams &M) {
    float sp, cp, st, ct;
    sincosf(phi, &sp, &cp);
    if (Q2D) {
        st = 1.0f;
        ct = 0.0f;
    } else {
        sincosf(theta, &st, &ct);
    }
    float n[3] = {st * cp, st * sp, ct};
    float dp[3] = {n[0], n[1], n[2]}, dn[3] = {0.f, 0.f, 0.f};
    const uint32_t mask = M.mask;
#pragma unroll
    for (int k = 0; k < 3; ++k) dp[k] += fld.flow(k);
    if (mask & M_MDD_FORCE) {
        float f[3];
        fld.gradb_dot(n, f);
#pragma unroll
        for (int k = 0; k < 3; ++k) dp[k] += f[k] * M.drag;
    }
    if (mask & M_EXTERNAL_FIELD) {
        float d = n[1] * M.reorient;
        dn[0] -= n[0] * d;
        dn[1] += M.reorient - n[1] * d;
        dn[2] -= n[2] * d;
    }
    if (mask & M_MDD_ROTATION) {
        float b[3] = {fld.b(0), fld.b(1), fld.b(2)};
        float d = n[0] * b[0] + n[1] * b[1] + n[2] * b[2];
#pragma unroll
        for (int k = 0; k < 3; ++k) dn[k] += b[k] - n[k] * d;
    }
    {
        float f[3];
        fld.vort_dot(n, f);
#pragma unroll
        for (int k = 0; k < 3; ++k) dn[k] -= f[k];
    }
    if (mask & M_JEFFREY_STRAIN) {
        float f[3];
        fld.strain_dot(n, f);
        float fn = M.shape * (f[0] * n[0] + f[1] * n[1] + f[2] * n[2]);
#pragma unroll
        for (int k = 0; k < 3; ++k) dn[k] += M.shape * f[k] - n[k] * fn;
    }
    const float diff = fld.diff();
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        dp[k] = dp[k] * M.dt + xi[k] * diff;
        dn[k] = dn[k] * M.dt;
    }
    // rotational diffusion about k perpendicular to n by rot (Rodrigues)
    float ax0 = cp * ct * sa - ca * sp, ax1 = ca * cp + ct * sa * sp, ax2 = -sa * st;
    float sr, cr;
    sincosf(rot, &sr, &cr);
    float cm1 = cr - 1.0f;
    dn[0] += n[0] * cm1 + (ax1 * n[2] - ax2 * n[1]) * sr;
    dn[1] += n[1] * cm1 + (ax2 * n[0] - ax0 * n[2]) * sr;
    dn[2] += n[2] * cm1 + (ax0 * n[1] - ax1 * n[0]) * sr;
    float v0 = n[0] + dn[0], v1 = n[1] + dn[1], v2 = n[2] + dn[2];
    float nphi = atan2f(v1, v0);
    step[0] = dp[0];
    step[1] = dp[1];
    step[2] = dp[2];
    if (Q2D) {
        phi = nphi < 0.0f ? nphi + 6.28318530717958647692f : nphi;
        theta = 1.57079632679489661923f;
    } else {
        // ang_pbc (src/particle.rs:37-44) of (nphi, nth): atan2f gives
        // nphi in [-pi, pi] and nth = pi/2 - atan2f(v2, |v_xy| >= 0) in
        // [0, pi], so modulo 2 pi is nphi + 2 pi for a negative nphi and the
        // identity otherwise, and the fold above pi cannot occur (fmodf, which
        // the general form would call, is far costlier on GB300).  A
        // non-finite angle stays non-finite, as through fmodf.
        const float nth = 1.57079632679489661923f - atan2f(v2, sqrtf(v0 * v0 + v1 * v1));
        if (nth > 3.14159265358979323846f) {
            float p = nphi + 3.14159265358979323846f;
            phi = p < 0.0f ? p + 6.28318530717958647692f : (p >= 6.28318530717958647692f ? p - 6.28318530717958647692f : p);
            theta = 6.28318530717958647692f - nth;
        } else {
            phi = nphi < 0.0f ? nphi + 6.28318530717958647692f : nphi;
            theta = nth;
        }
    }
}

// FP64 position advance: x + dx wrapped into [0, L) (modulo of
// src/particle.rs:26-35): one FP64 addition per coordinate; the wrap's range
// tests compare raw bits on the integer pipe and the rare wrap itself runs
// out of line (modulo_rare).
__device__ __forceinline__ double advance64(double x, float dx, double L) { return modulo_rare(x + f2d(dx), L); }

}  // namespace ss
