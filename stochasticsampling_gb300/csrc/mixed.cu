// mixed.cu -- the FP32 mixed-precision timestep (SS_FLAG_MIXED).
//
// Positions x, y, z stay FP64 and are accumulated in FP64.  Orientations,
// binning, the angular contraction, the FFTs, the k-space solve, the field
// table and the Langevin arithmetic are FP32.  The spectral solve keeps its
// k = 0 / mean handling in FP64: the per-component means of the stress and
// polarisation fields are summed in FP64 and removed before the FP32 FFT (so
// the transform only sees the fluctuations), and the mean dipolar field
// B_0 = <P> (the kept k = 0 mode, magnetic_solver.rs:88-94) is added back in
// FP64.  The mean flow is exactly zero (its k = 0 mode is multiplied by k).
//
// Layout: particles x, y, z f64 SoA + phi, theta f32 SoA (+ key, id as in the
// FP64 path); spectra float2; table rows of 16 (32 with dipolar terms) floats.
#include "kernels.cuh"
#include "mixed.cuh"
#include "mixed_device.cuh"

namespace ss {

// Particle::new in FP64, then the angles rounded to FP32 (and the position
// converted to fixed point when FIX); id (when given) gets the identity
template <bool FIX>
__global__ void k_ingest_m(const double *__restrict__ aos, unsigned long long n, DevParams P, double *__restrict__ x,
                           double *__restrict__ y, double *__restrict__ z, float *__restrict__ phi,
                           float *__restrict__ theta, uint32_t *__restrict__ id) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double *p = aos + 5 * i;
    double px = ref_modulo(p[0], P.bx), py = ref_modulo(p[1], P.by), pz = ref_modulo(p[2], P.bz);
    double ph = p[3], th = p[4];
    ref_ang_pbc(ph, th);
    px = ref_modulo(px, P.bx);
    py = ref_modulo(py, P.by);
    pz = ref_modulo(pz, P.bz);
    ref_ang_pbc(ph, th);
    if (FIX) {
        reinterpret_cast<unsigned long long *>(x)[i] = to_fixed(px, P.bx);
        reinterpret_cast<unsigned long long *>(y)[i] = to_fixed(py, P.by);
        reinterpret_cast<unsigned long long *>(z)[i] = to_fixed(pz, P.bz);
    } else {
        x[i] = px; y[i] = py; z[i] = pz;
    }
    phi[i] = (float)ph; theta[i] = (float)th;
    if (id) id[i] = (uint32_t)i;
}

template <bool FIX>
__global__ void k_egest_m(unsigned long long n, MixedParams M, const double *__restrict__ x,
                          const double *__restrict__ y, const double *__restrict__ z, const float *__restrict__ phi,
                          const float *__restrict__ theta, const uint32_t *__restrict__ id, double *__restrict__ aos) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double *p = aos + 5 * (unsigned long long)id[i];
    if (FIX) {
        p[0] = from_fixed(reinterpret_cast<const unsigned long long *>(x)[i], M.unit[0]);
        p[1] = from_fixed(reinterpret_cast<const unsigned long long *>(y)[i], M.unit[1]);
        p[2] = from_fixed(reinterpret_cast<const unsigned long long *>(z)[i], M.unit[2]);
    } else {
        p[0] = x[i]; p[1] = y[i]; p[2] = z[i];
    }
    p[3] = (double)phi[i]; p[4] = (double)theta[i];
}

template <bool FIX>
__device__ __forceinline__ void bin_any(const MixedParams &M, const double *x, const double *y, const double *z,
                                        unsigned long long i, float phi, float theta, uint32_t &cell,
                                        unsigned long long &bin) {
    if (FIX) {
        int ix = cell_fixed(reinterpret_cast<const unsigned long long *>(x)[i], M.gx);
        int iy = cell_fixed(reinterpret_cast<const unsigned long long *>(y)[i], M.gy);
        int iz = cell_fixed(reinterpret_cast<const unsigned long long *>(z)[i], M.gz);
        int ip = bin_f(phi, M.igwf[3], M.gphi);
        int it = bin_f(theta, M.igwf[4], M.gtheta);
        cell = (uint32_t)((ix * M.gy + iy) * M.gz + iz);
        bin = (unsigned long long)cell * (unsigned long long)M.nang + (unsigned long long)(ip * M.gtheta + it);
    } else {
        bin_mixed(M, x[i], y[i], z[i], phi, theta, cell, bin);
    }
}

template <bool FIX>
__global__ void k_bin_m(unsigned long long n, MixedParams M, const double *__restrict__ x,
                        const double *__restrict__ y, const double *__restrict__ z, const float *__restrict__ phi,
                        const float *__restrict__ theta, uint32_t *__restrict__ key, uint32_t *__restrict__ counts) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t cell;
    unsigned long long bin;
    bin_any<FIX>(M, x, y, z, i, phi[i], theta[i], cell, bin);
    atomicAdd(counts + bin, 1u);
    key[i] = cell;
}

// subtract the FP64 means before the FP32 transform
__global__ void k_center_m(float *__restrict__ fr, int c0, int c1, int ncell, int cstride,
                           const double *__restrict__ sums) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    long long total = (long long)(c1 - c0) * ncell;
    if (i >= total) return;
    int comp = c0 + (int)(i / ncell);
    long long idx = (long long)comp * cstride + (i % ncell);
    float mean = (float)(sums[comp] / (double)ncell);
    fr[idx] -= mean;
}

// the operators of the FP64 path's k_kspace (kernels.cu) in FP32
__device__ __forceinline__ void flow_ops_f(const float k[3], const float kn[3], float fac, const float2 *sig,
                                           float2 *o) {
    float2 sg[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        const float2 a0 = sig[3 * r + 0], a1 = sig[3 * r + 1], a2 = sig[3 * r + 2];
        sg[r].x = a0.x * k[0] + a1.x * k[1] + a2.x * k[2];
        sg[r].y = a0.y * k[0] + a1.y * k[1] + a2.y * k[2];
    }
    const float ksr = kn[0] * sg[0].x + kn[1] * sg[1].x + kn[2] * sg[2].x;
    const float ksi = kn[0] * sg[0].y + kn[1] * sg[1].y + kn[2] * sg[2].y;
    float2 u[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        const float tr = (sg[r].x - kn[r] * ksr) * fac;
        const float ti = (sg[r].y - kn[r] * ksi) * fac;
        u[r] = make_float2(-ti, tr);
        o[9 + r] = u[r];
    }
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) o[3 * a + b] = make_float2(-(k[a] * u[b].y), k[a] * u[b].x);
}

__device__ __forceinline__ void mag_ops_f(const float k[3], const float kn[3], float norm, bool kzero,
                                          const float2 *p, float2 *o) {
    const float dr = kn[0] * p[0].x + kn[1] * p[1].x + kn[2] * p[2].x;
    const float di = kn[0] * p[0].y + kn[1] * p[1].y + kn[2] * p[2].y;
    float2 b[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        // the k = 0 mode (the mean) was removed and is added back in FP64
        b[r] = kzero ? make_float2(0.f, 0.f)
                     : make_float2((p[r].x - kn[r] * dr) / norm, (p[r].y - kn[r] * di) / norm);
        o[9 + r] = b[r];
    }
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int bb = 0; bb < 3; ++bb) o[3 * a + bb] = make_float2(-(k[a] * b[bb].y), k[a] * b[bb].x);
}

// the half-spectrum k space of the FP64 path (kernels.cu, k_kspace) in FP32:
// the operators' Hermitian part (ANTI: the anti-Hermitian part), evaluated
// twice only on Nyquist planes
template <bool FLOW, bool MAG, bool ANTI>
__global__ void k_kspace_m(const float2 *__restrict__ fwd, float2 *__restrict__ out, MixedParams M, float screening,
                           float stepx, float stepy, float stepz) {
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    const int nh = M.nhalf;
    if (h >= nh) return;
    const int iz = h % M.hdim[2];
    const int iy = (h / M.hdim[2]) % M.hdim[1];
    const int ix = h / (M.hdim[2] * M.hdim[1]);
    const float k[3] = {kval_f(ix, M.gx, stepx), kval_f(iy, M.gy, stepy), kval_f(iz, M.gz, stepz)};
    const bool nyq[3] = {(M.gx & 1) == 0 && 2 * ix == M.gx, (M.gy & 1) == 0 && 2 * iy == M.gy,
                         (M.gz & 1) == 0 && 2 * iz == M.gz};
    const bool mirror = nyq[0] || nyq[1] || nyq[2];
    const bool kzero = (ix | iy | iz) == 0;
    const float s = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
    const float ik2 = kzero ? 0.f : 1.f / s;
    const float inrm = kzero ? 0.f : rsqrtf(s);
    const float kn[3] = {k[0] * inrm, k[1] * inrm, k[2] * inrm};
    const float km[3] = {nyq[0] ? k[0] : -k[0], nyq[1] ? k[1] : -k[1], nyq[2] ? k[2] : -k[2]};
    const float knm[3] = {km[0] * inrm, km[1] * inrm, km[2] * inrm};
    const float norm = (float)M.ncell;
    auto emit = [&](int c0, const float2 *X, const float2 *Xm) {
#pragma unroll
        for (int j = 0; j < 12; ++j) {
            float2 v;
            if (!mirror) v = ANTI ? make_float2(0.f, 0.f) : X[j];
            else if (ANTI) v = make_float2((X[j].y + Xm[j].y) * 0.5f, -(X[j].x - Xm[j].x) * 0.5f);
            else v = make_float2((X[j].x + Xm[j].x) * 0.5f, (X[j].y - Xm[j].y) * 0.5f);
            out[(long long)(c0 + j) * nh + h] = v;
        }
    };
    if (FLOW) {
        float2 sig[9], X[12], Xm[12];
#pragma unroll
        for (int j = 0; j < 9; ++j) sig[j] = fwd[(long long)j * nh + h];
        const float fac = (ik2 + screening) / norm;
        flow_ops_f(k, kn, fac, sig, X);
        if (mirror) {
#pragma unroll
            for (int j = 0; j < 9; ++j) sig[j].y = -sig[j].y;
            flow_ops_f(km, knm, fac, sig, Xm);
        }
        emit(0, X, Xm);
    }
    if (MAG) {
        float2 pol[3], X[12], Xm[12];
#pragma unroll
        for (int j = 0; j < 3; ++j) pol[j] = fwd[(long long)(9 + j) * nh + h];
        mag_ops_f(k, kn, norm, kzero, pol, X);
        if (mirror) {
#pragma unroll
            for (int j = 0; j < 3; ++j) pol[j].y = -pol[j].y;
            mag_ops_f(km, knm, norm, kzero, pol, Xm);
        }
        emit(12, X, Xm);
    }
}

template <bool FLOW, bool MAG>
__global__ void k_table_m(const float *__restrict__ inv, MixedParams M, float *__restrict__ table, int tstride,
                          const double *__restrict__ sums) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int nc = M.ncell;
    if (c >= nc) return;
    float *row = table + (long long)c * tstride;
    if (FLOW) {
        float g[9];
#pragma unroll
        for (int j = 0; j < 9; ++j) g[j] = inv[(long long)j * nc + c];
#pragma unroll
        for (int r = 0; r < 3; ++r) row[T_U + r] = inv[(long long)(9 + r) * nc + c];
        row[T_W01] = (g[1] - g[3]) * 0.5f;
        row[T_W02] = (g[2] - g[6]) * 0.5f;
        row[T_W12] = (g[5] - g[7]) * 0.5f;
        row[T_E00] = g[0];
        row[T_E01] = (g[1] + g[3]) * 0.5f;
        row[T_E02] = (g[2] + g[6]) * 0.5f;
        row[T_E11] = g[4];
        row[T_E12] = (g[5] + g[7]) * 0.5f;
        row[T_E22] = g[8];
    }
    if (MAG) {
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            double b = (double)inv[(long long)(21 + r) * nc + c] + sums[9 + r] / (double)nc;
            row[T_B + r] = (float)(b * M.mdd);
        }
#pragma unroll
        for (int j = 0; j < 9; ++j) row[T_GB + j] = inv[(long long)(12 + j) * nc + c];
    }
}

// complex double fields for the FP64 getters from FP32 real and imaginary
// parts; adds the FP64 mean back to the components listed in [m0, m1)
__global__ void k_widen_m(const float *__restrict__ re, const float *__restrict__ im, long long count, int ncell,
                          int comp0, int m0, int m1, const double *__restrict__ sums, double2 *__restrict__ dst) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= count) return;
    int comp = comp0 + (int)(i / ncell);
    double r = (double)re[i];
    if (comp >= m0 && comp < m1) r += sums[comp - 12] / (double)ncell;
    dst[i] = make_double2(r, im ? (double)im[i] : 0.0);
}

__global__ void k_real_to_complex_f(const float *__restrict__ src, int count, int sstride, float2 *__restrict__ dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) dst[i] = make_float2(src[(long long)i * sstride], 0.f);
}
__global__ void k_complex_to_real_f(const float2 *__restrict__ src, int count, float *__restrict__ dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) dst[i] = src[i].x;
}

// NOISE: 0 Philox, 1 host array.  CANON (quasi2d only): z == 0 and
// theta == pi/2 already hold, so they are neither read nor written.  FIX:
// positions in 64-bit fixed point.  Two entry points: k_update_m (quasi-2-D)
// and k_update_m3 (3-D), the latter held to 48 registers (5 blocks of 256
// per SM, no spills): latency bound, it gains from the extra warps (update
// 0.69 -> 0.61 ms on the 3-D workload), where the quasi-2-D forms lose 12 %
// under any explicit minimum of blocks.
template <bool Q2D, bool CANON, bool MAG, int NOISE, bool FIX>
__device__ __forceinline__ void update_m_body(const MixedParams &M, double *__restrict__ x, double *__restrict__ y,
                                              double *__restrict__ z, float *__restrict__ phi,
                                              float *__restrict__ theta, uint32_t *__restrict__ key,
                                              const uint32_t *__restrict__ id, const float *__restrict__ table,
                                              const double *__restrict__ noise,
                                              const unsigned long long *__restrict__ d_step,
                                              uint32_t *__restrict__ counts_next) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i >= M.n) return;
    const int ts = MAG ? TABLE_STRIDE_MAG : TABLE_STRIDE;
    uint32_t cell = key[i];
    float pph = phi[i], pth = 1.57079632679489661923f;
    if (!CANON) pth = theta[i];
    TableFieldsF F(table + (long long)cell * ts);
    float xi[3], ca, sa, rot;
    // the noise is keyed by the caller's index of the particle (rows are sorted by cell at ingest)
    const uint32_t pid = id[i];
    if (NOISE == 0) {
        philox_noise_f<Q2D>(M.seed, pid, *d_step, M.sigma_rot, xi, ca, sa, rot);
    } else {
        const double *r = noise + 5ull * pid;
        xi[0] = (float)r[0]; xi[1] = (float)r[1]; xi[2] = (float)r[2];
        sincosf((float)r[3], &sa, &ca);
        rot = (float)r[4];
    }
    float st[3];
    if (Q2D && !CANON) {
        // first step after init: theta may differ from pi/2
        langevin_mixed<false>(pph, pth, st, F, xi, ca, sa, rot, M);
        pth = 1.57079632679489661923f;
    } else {
        langevin_mixed<Q2D>(pph, pth, st, F, xi, ca, sa, rot, M);
    }
    uint32_t ncell;
    unsigned long long bin;
    if (FIX) {
        unsigned long long *X = reinterpret_cast<unsigned long long *>(x);
        unsigned long long *Y = reinterpret_cast<unsigned long long *>(y);
        unsigned long long *Z = reinterpret_cast<unsigned long long *>(z);
        unsigned long long px = X[i] + step_fixed(st[0], M.s32[0]);
        unsigned long long py = Y[i] + step_fixed(st[1], M.s32[1]);
        unsigned long long pz = 0ull;
        if (!Q2D) pz = Z[i] + step_fixed(st[2], M.s32[2]);
        int ix = cell_fixed(px, M.gx), iy = cell_fixed(py, M.gy), iz = Q2D ? 0 : cell_fixed(pz, M.gz);
        int ip = bin_f(pph, M.igwf[3], M.gphi), it = bin_f(pth, M.igwf[4], M.gtheta);
        ncell = (uint32_t)((ix * M.gy + iy) * M.gz + iz);
        bin = (unsigned long long)ncell * (unsigned long long)M.nang + (unsigned long long)(ip * M.gtheta + it);
        X[i] = px;
        Y[i] = py;
        if (!CANON) Z[i] = pz;
    } else {
        double px = advance64(x[i], st[0], M.bx);
        double py = advance64(y[i], st[1], M.by);
        double pz = 0.0;
        if (!Q2D) pz = advance64(z[i], st[2], M.bz);
        bin_mixed(M, px, py, pz, pph, pth, ncell, bin);
        x[i] = px;
        y[i] = py;
        if (!CANON) z[i] = pz;
    }
    atomicAdd(counts_next + bin, 1u);
    key[i] = ncell;
    phi[i] = pph;
    if (!CANON) theta[i] = pth;
}
#define SS_UPDATE_M_ARGS                                                                                           \
    MixedParams M, double *__restrict__ x, double *__restrict__ y, double *__restrict__ z, float *__restrict__ phi, \
        float *__restrict__ theta, uint32_t *__restrict__ key, const uint32_t *__restrict__ id,                   \
        const float *__restrict__ table, const double *__restrict__ noise,                                         \
        const unsigned long long *__restrict__ d_step, uint32_t *__restrict__ counts_next
template <bool CANON, bool MAG, int NOISE, bool FIX>
__global__ void __launch_bounds__(256) k_update_m(SS_UPDATE_M_ARGS) {
    update_m_body<true, CANON, MAG, NOISE, FIX>(M, x, y, z, phi, theta, key, id, table, noise, d_step, counts_next);
}
template <bool MAG, int NOISE, bool FIX>
__global__ void __launch_bounds__(256, 5) k_update_m3(SS_UPDATE_M_ARGS) {
    update_m_body<false, false, MAG, NOISE, FIX>(M, x, y, z, phi, theta, key, id, table, noise, d_step, counts_next);
}
#undef SS_UPDATE_M_ARGS

template <bool Q2D>
__global__ void k_noise_m(MixedParams M, unsigned long long t, double *__restrict__ out) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i >= M.n) return;
    float xi[3], ca, sa, rot;
    philox_noise_f<Q2D>(M.seed, (uint32_t)i, t, M.sigma_rot, xi, ca, sa, rot);
    double *r = out + 5 * i;
    r[0] = xi[0]; r[1] = xi[1]; r[2] = xi[2]; r[3] = atan2((double)sa, (double)ca); r[4] = rot;
    if (r[3] < 0.0) r[3] += kTwoPi;
}

// ---- periodic re-sort of the resident particles by cell ------------------
// Rows sorted by cell at ingest keep the particles of a cell together for
// many steps, but they drift (on the 3-D workload the update is 10 % slower
// after 3,000 steps).  A counting sort on the cell keys the update wrote:
// the particles per cell (warp-aggregated atomics), an exclusive scan, and a
// scatter of every row into the other buffer set at cursor[key] + its rank.
// The order within a cell follows the atomics, which changes no result: the
// noise is keyed by the particle's caller index, the histogram is integer
// counts, and the rows go back to the caller by that index.
__global__ void k_count_keys(const uint32_t *__restrict__ key, unsigned long long n, uint32_t *__restrict__ cellcount) {
    const unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t k = key[i];
    const unsigned same = __match_any_sync(__activemask(), k);
    if ((int)(threadIdx.x & 31) == __ffs(same) - 1) atomicAdd(cellcount + k, (uint32_t)__popc(same));
}
// positions as 64-bit words (FP64 or fixed point alike), angles FP32
__global__ void __launch_bounds__(256) k_scatter_m(unsigned long long n, const unsigned long long *__restrict__ x,
                                                   const unsigned long long *__restrict__ y,
                                                   const unsigned long long *__restrict__ z,
                                                   const float *__restrict__ phi, const float *__restrict__ theta,
                                                   const uint32_t *__restrict__ key, const uint32_t *__restrict__ id,
                                                   unsigned long long *__restrict__ x2, unsigned long long *__restrict__ y2,
                                                   unsigned long long *__restrict__ z2, float *__restrict__ phi2,
                                                   float *__restrict__ theta2, uint32_t *__restrict__ key2,
                                                   uint32_t *__restrict__ id2, uint32_t *__restrict__ cursor) {
    const unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int lane = threadIdx.x & 31;
    const uint32_t k = key[i];
    const unsigned same = __match_any_sync(__activemask(), k);
    const int leader = __ffs(same) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(cursor + k, (uint32_t)__popc(same));
    base = __shfl_sync(same, base, leader);
    const uint32_t dst = base + (uint32_t)__popc(same & ((1u << lane) - 1u));
    x2[dst] = x[i];
    y2[dst] = y[i];
    z2[dst] = z[i];
    phi2[dst] = phi[i];
    theta2[dst] = theta[i];
    key2[dst] = k;
    id2[dst] = id[i];
}

// ========================================================================
static inline unsigned nb(unsigned long long n, unsigned bs) { return (unsigned)((n + bs - 1) / bs); }

void launch_ingest_m(cudaStream_t s, bool fixed, const double *aos, unsigned long long n, const DevParams &P,
                     const MixedParams &M, double *const xs[3], float *const as[2], uint32_t *id) {
    (void)M;
    if (!n) return;
    if (fixed) k_ingest_m<true><<<nb(n, 256), 256, 0, s>>>(aos, n, P, xs[0], xs[1], xs[2], as[0], as[1], id);
    else k_ingest_m<false><<<nb(n, 256), 256, 0, s>>>(aos, n, P, xs[0], xs[1], xs[2], as[0], as[1], id);
}
void launch_egest_m(cudaStream_t s, bool fixed, unsigned long long n, const MixedParams &M, double *const xs[3],
                    float *const as[2], const uint32_t *id, double *aos) {
    if (!n) return;
    if (fixed) k_egest_m<true><<<nb(n, 256), 256, 0, s>>>(n, M, xs[0], xs[1], xs[2], as[0], as[1], id, aos);
    else k_egest_m<false><<<nb(n, 256), 256, 0, s>>>(n, M, xs[0], xs[1], xs[2], as[0], as[1], id, aos);
}
void launch_bin_m(cudaStream_t s, bool fixed, unsigned long long n, const MixedParams &M, double *const xs[3],
                  float *const as[2], uint32_t *key, uint32_t *counts) {
    if (!n) return;
    if (fixed) k_bin_m<true><<<nb(n, 256), 256, 0, s>>>(n, M, xs[0], xs[1], xs[2], as[0], as[1], key, counts);
    else k_bin_m<false><<<nb(n, 256), 256, 0, s>>>(n, M, xs[0], xs[1], xs[2], as[0], as[1], key, counts);
}
// counts -> the denoiser's input, counts / (N / nbins) (mean 1)
__global__ void k_counts_to_unit(const uint32_t *__restrict__ counts, long long nbins, float inv_mean,
                                 float *__restrict__ x) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < nbins) x[i] = (float)counts[i] * inv_mean;
}
void launch_counts_to_unit(cudaStream_t s, const uint32_t *counts, long long nbins, float inv_mean, float *x) {
    if (nbins > 0) k_counts_to_unit<<<nb((unsigned long long)nbins, 256), 256, 0, s>>>(counts, nbins, inv_mean, x);
}
void launch_center_m(cudaStream_t s, float *fr, int c0, int c1, int ncell, int cstride, const double *sums) {
    long long total = (long long)(c1 - c0) * ncell;
    if (total > 0) k_center_m<<<nb(total, 256), 256, 0, s>>>(fr, c0, c1, ncell, cstride, sums);
}
void launch_kspace_m(cudaStream_t s, bool flow, bool mag, bool anti, const float2 *fwd, float2 *inv,
                     const MixedParams &M, float screening) {
    float sx = (float)(kTwoPi / M.bx), sy = (float)(kTwoPi / M.by), sz = (float)(kTwoPi / M.bz);
    unsigned b = nb(M.nhalf, 128);
#define SS_KSM(F, G)                                                                                     \
    do {                                                                                                 \
        if (anti) k_kspace_m<F, G, true><<<b, 128, 0, s>>>(fwd, inv, M, screening, sx, sy, sz);      \
        else k_kspace_m<F, G, false><<<b, 128, 0, s>>>(fwd, inv, M, screening, sx, sy, sz);          \
    } while (0)
    if (flow && mag) SS_KSM(true, true);
    else if (flow) SS_KSM(true, false);
    else SS_KSM(false, true);
#undef SS_KSM
}
void launch_table_m(cudaStream_t s, bool flow, bool mag, const float *inv, const MixedParams &M, float *table,
                    int tstride, const double *sums) {
    unsigned b = nb(M.ncell, 128);
    if (flow && mag) k_table_m<true, true><<<b, 128, 0, s>>>(inv, M, table, tstride, sums);
    else if (flow) k_table_m<true, false><<<b, 128, 0, s>>>(inv, M, table, tstride, sums);
    else k_table_m<false, true><<<b, 128, 0, s>>>(inv, M, table, tstride, sums);
}
void launch_widen_m(cudaStream_t s, const float *re, const float *im, long long count, int ncell, int comp0, int m0,
                    int m1, const double *sums, double2 *dst) {
    if (count > 0) k_widen_m<<<nb(count, 256), 256, 0, s>>>(re, im, count, ncell, comp0, m0, m1, sums, dst);
}
void launch_real_to_complex_f(cudaStream_t s, const float *src, int count, int sstride, float2 *dst) {
    if (count > 0) k_real_to_complex_f<<<nb(count, 128), 128, 0, s>>>(src, count, sstride, dst);
}
void launch_complex_to_real_f(cudaStream_t s, const float2 *src, int count, float *dst) {
    if (count > 0) k_complex_to_real_f<<<nb(count, 128), 128, 0, s>>>(src, count, dst);
}
void launch_update_m(cudaStream_t s, bool fixed, bool q2d, bool canon, bool mag, bool host_noise, const MixedParams &M,
                     double *const xs[3], float *const as[2], uint32_t *key, const uint32_t *id, const float *table,
                     const double *noise, const unsigned long long *d_step, uint32_t *counts_next) {
    if (!M.n) return;
    unsigned b = nb(M.n, 256);
#define SS_UPDM(K, ...)                                                                                     \
    do {                                                                                                    \
        if (fixed)                                                                                          \
            K<__VA_ARGS__, true><<<b, 256, 0, s>>>(M, xs[0], xs[1], xs[2], as[0], as[1], key, id, table,   \
                                                   noise, d_step, counts_next);                             \
        else                                                                                                \
            K<__VA_ARGS__, false><<<b, 256, 0, s>>>(M, xs[0], xs[1], xs[2], as[0], as[1], key, id, table,  \
                                                    noise, d_step, counts_next);                            \
    } while (0)
#define SS_UPDM2(C, G) \
    do { if (host_noise) SS_UPDM(k_update_m, C, G, 1); else SS_UPDM(k_update_m, C, G, 0); } while (0)
#define SS_UPDM3(G) \
    do { if (host_noise) SS_UPDM(k_update_m3, G, 1); else SS_UPDM(k_update_m3, G, 0); } while (0)
    if (q2d) {
        if (canon) { if (mag) SS_UPDM2(true, true); else SS_UPDM2(true, false); }
        else { if (mag) SS_UPDM2(false, true); else SS_UPDM2(false, false); }
    } else {
        if (mag) SS_UPDM3(true); else SS_UPDM3(false);
    }
#undef SS_UPDM3
#undef SS_UPDM2
#undef SS_UPDM
}
void launch_resort_m(cudaStream_t s, const MixedParams &M, double *const xs[3], float *const as[2], const uint32_t *key,
                     const uint32_t *id, double *const xd[3], float *const ad[2], uint32_t *keyd, uint32_t *idd,
                     uint32_t *cellcount, uint32_t *cursor) {
    if (!M.n) return;
    launch_zero_u32(s, cellcount, M.ncell);
    k_count_keys<<<nb(M.n, 256), 256, 0, s>>>(key, M.n, cellcount);
    launch_scan(s, cellcount, M.ncell, cursor);
    auto w = [](double *p) { return reinterpret_cast<unsigned long long *>(p); };
    k_scatter_m<<<nb(M.n, 256), 256, 0, s>>>(M.n, w(xs[0]), w(xs[1]), w(xs[2]), as[0], as[1], key, id, w(xd[0]),
                                              w(xd[1]), w(xd[2]), ad[0], ad[1], keyd, idd, cursor);
}
void launch_noise_m(cudaStream_t s, bool q2d, const MixedParams &M, unsigned long long t, double *out) {
    if (!M.n) return;
    if (q2d) k_noise_m<true><<<nb(M.n, 256), 256, 0, s>>>(M, t, out);
    else k_noise_m<false><<<nb(M.n, 256), 256, 0, s>>>(M, t, out);
}

}  // namespace ss
