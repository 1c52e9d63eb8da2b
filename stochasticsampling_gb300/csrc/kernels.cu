// kernels.cu -- the timestep kernels (sm_103a) and their launch wrappers.
//
// Step pipeline (one simulation, all on one stream):
//   contract  counts -> stress sigma_ij, polarisation P_c (complex, im = 0),
//             per-cell diffusion length, particles per cell
//   [sort]    counting sort of the particle arrays by spatial cell
//   cuFFT     forward Z2Z of 9 (+3) components
//   kspace    Oseen projection + screening, dipolar projection, gradients
//   cuFFT     inverse Z2Z of 12 (+12) components
//   table     per-cell row: Re u, W, E, B*mdd, grad B
//   update    gather row by cell, Langevin step, wrap, bin into next histogram
#include "f32x2.cuh"
#include "kernels.cuh"

#include <cstdio>

namespace ss {

// ------------------------------------------------------------------------
// small helpers
// ------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ uint32_t warp_sum_u(uint32_t v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// k value of FFT index i on an axis of n cells and box length L:
// get_k_sampling (src/mesh/fft_helper.rs:26-51): index i < ceil(n/2) -> i,
// else i - n (the Nyquist mode of an even n is negative), times 2 pi / L.
__device__ __forceinline__ double kval(int i, int n, double step) {
    int b = (n % 2 == 0) ? n / 2 : n / 2 + 1;
    return (double)(i < b ? i : i - n) * step;
}

// ------------------------------------------------------------------------
// particle ingest / egest / binning
// ------------------------------------------------------------------------

// Validation of caller rows [n][5] on the device (integer tests on the bits):
// scan[0] = the first particle with a non-finite coordinate (atomicMin; left
// at ~0 when there is none), scan[1] |= 1 when a particle is outside the
// canonical quasi2d state z = 0, theta = pi/2.
__global__ void k_scan_rows(const double *__restrict__ aos, unsigned long long n,
                            unsigned long long *__restrict__ scan) {
    const unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    bool bad = false, noncanon = false;
    if (i < n) {
        const unsigned long long *b = reinterpret_cast<const unsigned long long *>(aos + 5 * i);
#pragma unroll
        for (int k = 0; k < 5; ++k) bad |= ((b[k] >> 52) & 0x7FFull) == 0x7FFull;
        const unsigned long long half_pi = (unsigned long long)__double_as_longlong(kPiHalf);
        noncanon = b[2] != 0ull || b[4] != half_pi;  // z == +0.0 (the value a quasi2d step writes)
    }
    if (bad) atomicMin(&scan[0], i);
    if (__any_sync(0xffffffffu, noncanon) && (threadIdx.x & 31) == 0) atomicOr(&scan[1], 1ull);
}

// Particle::new (src/particle.rs:186-201) on one caller row: modulo on the
// positions and ang_pbc on the angles, then both once more.
__device__ __forceinline__ void ingest_row(const double *__restrict__ p, const DevParams &P, double &px, double &py,
                                           double &pz, double &ph, double &th) {
    px = ref_modulo(p[0], P.bx);
    py = ref_modulo(p[1], P.by);
    pz = ref_modulo(p[2], P.bz);
    ph = p[3];
    th = p[4];
    ref_ang_pbc(ph, th);
    px = ref_modulo(px, P.bx);
    py = ref_modulo(py, P.by);
    pz = ref_modulo(pz, P.bz);
    ref_ang_pbc(ph, th);
}

// Rows reordered by spatial cell before the ingest (a counting sort), so
// that the particles of a cell sit together in memory: the update's field
// gathers and histogram atomics then hit the same rows one after another
// (the 3-D histogram of 2^25 bins does not fit L2).  Particles move a
// fraction of a cell per step, so the order keeps its locality; the noise
// stays keyed by the caller's index (id).  The key is the cell of the
// wrapped position from an FP32 estimate; the exact bins come later.
__global__ void k_row_cells(const double *__restrict__ aos, unsigned long long n, DevParams P,
                            uint32_t *__restrict__ cellkey, uint32_t *__restrict__ cellcount) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double *p = aos + 5 * i;
    const int nk[3] = {P.gx, P.gy, P.gz};
    const double L[3] = {P.bx, P.by, P.bz};
    int c[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int f = (int)floorf(d2f_pos(ref_modulo(p[k], L[k])) * P.igwf[k]);
        c[k] = f < 0 ? 0 : (f >= nk[k] ? nk[k] - 1 : f);
    }
    const uint32_t cell = (uint32_t)((c[0] * P.gy + c[1]) * P.gz + c[2]);
    cellkey[i] = cell;
    atomicAdd(cellcount + cell, 1u);
}
__global__ void k_sort_rows(const double *__restrict__ aos, unsigned long long n, const uint32_t *__restrict__ cellkey,
                            uint32_t *__restrict__ cursor, double *__restrict__ sorted, uint32_t *__restrict__ orig) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned long long pos = atomicAdd(cursor + cellkey[i], 1u);
    const double *src = aos + 5 * i;
    double *dst = sorted + 5 * pos;
#pragma unroll
    for (int k = 0; k < 5; ++k) dst[k] = src[k];
    orig[pos] = (uint32_t)i;
}

// SoA slot i -> AoS row id[i] (the caller's order)
__global__ void k_egest(unsigned long long n, const double *__restrict__ x, const double *__restrict__ y,
                        const double *__restrict__ z, const double *__restrict__ phi,
                        const double *__restrict__ theta, const uint32_t *__restrict__ id,
                        double *__restrict__ aos) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double *p = aos + 5 * (unsigned long long)id[i];
    p[0] = x[i]; p[1] = y[i]; p[2] = z[i]; p[3] = phi[i]; p[4] = theta[i];
}

// CANON: z == 0 and theta == pi/2 (every particle after a quasi2d step), so
// their bins are 0 and the precomputed bin of pi/2.
template <bool CANON = false>
__device__ __forceinline__ void bin_particle(const DevParams &P, double x, double y, double z, double phi,
                                             double theta, uint32_t &cell, unsigned long long &bin,
                                             uint32_t &err) {
    int ix = ref_bin_f(x, P.gw[0], P.igw[0], P.igwf[0], P.bintol[0], P.gx, err);
    int iy = ref_bin_f(y, P.gw[1], P.igw[1], P.igwf[1], P.bintol[1], P.gy, err);
    int iz = CANON ? 0 : ref_bin_f(z, P.gw[2], P.igw[2], P.igwf[2], P.bintol[2], P.gz, err);
    int ip = ref_bin_f(phi, P.gw[3], P.igw[3], P.igwf[3], P.bintol[3], P.gphi, err);
    int it = CANON ? P.bin_theta_half : ref_bin_f(theta, P.gw[4], P.igw[4], P.igwf[4], P.bintol[4], P.gtheta, err);
    cell = (uint32_t)((ix * P.gy + iy) * P.gz + iz);
    bin = (unsigned long long)cell * (unsigned long long)P.nang + (unsigned long long)(ip * P.gtheta + it);
}

// Particle::new (ingest_row, AoS [n][5] -> SoA) fused with the first
// histogram, Distribution::histogram_from (src/distribution/mod.rs:146-160)
// with integer counts, and each particle's spatial cell (Simulation::init,
// src/bin/simulation/mod.rs:163-196): one pass over the rows.  CANON: every
// row in the canonical quasi-2-D state.
template <bool CANON>
__global__ void k_ingest_bin(const double *__restrict__ aos, unsigned long long n, DevParams P,
                             double *__restrict__ x, double *__restrict__ y, double *__restrict__ z,
                             double *__restrict__ phi, double *__restrict__ theta, uint32_t *__restrict__ id,
                             uint32_t *__restrict__ key, uint32_t *__restrict__ counts,
                             uint32_t *__restrict__ errflag) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double px, py, pz, ph, th;
    ingest_row(aos + 5 * i, P, px, py, pz, ph, th);
    x[i] = px; y[i] = py; z[i] = pz; phi[i] = ph; theta[i] = th;
    if (id) id[i] = (uint32_t)i;
    uint32_t err = 0, cell;
    unsigned long long bin;
    bin_particle<CANON>(P, px, py, pz, ph, th, cell, bin, err);
    atomicAdd(counts + bin, 1u);
    key[i] = cell;
    if (err) atomicOr(errflag, err);
}

// k_ingest_bin with the row checks of k_scan_rows, for rows off .. off + n
// of a larger array (aos, the arrays and id point at row off): scan[0] gets
// the first row with a non-finite coordinate, scan[1] a non-zero value when
// some row is off the canonical quasi-2-D state.  Rows with a non-finite
// coordinate are binned like any other (their bins clamp, nothing is
// flagged); the caller discards the whole result when scan[0] is set.
__global__ void k_ingest_bin_check(const double *__restrict__ aos, unsigned long long n, unsigned long long off,
                                   DevParams P, double *__restrict__ x, double *__restrict__ y,
                                   double *__restrict__ z, double *__restrict__ phi, double *__restrict__ theta,
                                   uint32_t *__restrict__ id, uint32_t *__restrict__ key,
                                   uint32_t *__restrict__ counts, unsigned long long *__restrict__ scan,
                                   uint32_t *__restrict__ errflag) {
    const unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    bool noncanon = false;
    if (i < n) {
        const double *p = aos + 5 * i;
        const unsigned long long *b = reinterpret_cast<const unsigned long long *>(p);
        bool bad = false;
#pragma unroll
        for (int k = 0; k < 5; ++k) bad |= ((b[k] >> 52) & 0x7FFull) == 0x7FFull;
        noncanon = b[2] != 0ull || b[4] != (unsigned long long)__double_as_longlong(kPiHalf);
        if (bad) atomicMin(&scan[0], off + i);
        double px, py, pz, ph, th;
        ingest_row(p, P, px, py, pz, ph, th);
        x[i] = px; y[i] = py; z[i] = pz; phi[i] = ph; theta[i] = th;
        id[i] = (uint32_t)(off + i);
        uint32_t err = 0, cell;
        unsigned long long bin;
        bin_particle<false>(P, px, py, pz, ph, th, cell, bin, err);
        atomicAdd(counts + bin, 1u);
        key[i] = cell;
        if (err && !bad) atomicOr(errflag, err);
    }
    if (__any_sync(0xffffffffu, noncanon) && (threadIdx.x & 31) == 0) atomicOr(&scan[1], 1ull);
}

// counts -> normalised distribution, (c / D) * V exactly as
// sample_from + the box-volume rescale (distribution/mod.rs:183,
// simulation/mod.rs:255-257)
__global__ void k_counts_to_dist(const uint32_t *__restrict__ counts, long long nbins, DevParams P,
                                 double *__restrict__ dist) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= nbins) return;
    dist[i] = ((double)counts[i] / P.dist_den) * P.volume;
}

// ------------------------------------------------------------------------
// angular contraction: average_stress (src/flowfield/stress.rs:60-96),
// DirectorField::from_distribution (src/polarization/director.rs:36-61) and
// the density of src/bin/simulation/mod.rs:312-316.  One thread per cell runs
// over that cell's angle row (one cache line per thread for 32 angles,
// reused from L1), with the angle kernels broadcast from shared memory; the
// sums run in angle order, like sum_axis.  kern rows: 0..8 stress kernel
// K_ij, 9..11 orientation kernel n_c.
// ------------------------------------------------------------------------
template <bool STRESS, bool MAG, bool FROM_DIST, bool SMEM>
__global__ void __launch_bounds__(64) k_contract(const uint32_t *__restrict__ counts,
                                                 const double *__restrict__ dist,
                                                 const double *__restrict__ lut, int lut_n,
                                                 const double *__restrict__ kern, DevParams P,
                                                 double *__restrict__ fwd, double *__restrict__ table,
                                                 int tstride, uint32_t *__restrict__ cellcount) {
    extern __shared__ double sk[];
    const int na = P.nang;
    if (SMEM) {
        for (int i = threadIdx.x; i < 12 * na; i += blockDim.x) sk[i] = kern[i];
        __syncthreads();
    }
    const double *K = SMEM ? sk : kern;
    int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= P.ncell) return;
    double acc[13];
#pragma unroll
    for (int j = 0; j < 13; ++j) acc[j] = 0.0;
    uint32_t csum = 0;
    const long long row = (long long)cell * na;
    for (int a = 0; a < na; ++a) {
        double f;
        if (FROM_DIST) {
            f = dist[row + a];
        } else {
            uint32_t c = counts[row + a];
            csum += c;
            f = ((int)c < lut_n) ? __ldg(lut + c) : ((double)c / P.dist_den) * P.volume;
        }
        if (STRESS) {
#pragma unroll
            for (int j = 0; j < 9; ++j) acc[j] = fma(K[j * na + a], f, acc[j]);
        }
        if (MAG) {
#pragma unroll
            for (int j = 9; j < 12; ++j) acc[j] = fma(K[j * na + a], f, acc[j]);
        }
        acc[12] += f;
    }
    if (STRESS) {
#pragma unroll
        for (int j = 0; j < 9; ++j) fwd[(long long)j * P.cstride + cell] = acc[j] * P.measure;
    }
    if (MAG) {
#pragma unroll
        for (int j = 0; j < 3; ++j) fwd[(long long)(9 + j) * P.cstride + cell] = acc[9 + j] * P.measure;
    }
    double dens = acc[12] * P.dthph;
    double volex = P.volex * dens;
    table[(long long)cell * tstride + T_DIFF] = sqrt(2.0 * P.dt * (P.Dt + volex));
    if (tstride == TABLE_STRIDE_MAG) table[(long long)cell * tstride + T_DENS] = dens;
    if (!FROM_DIST) cellcount[cell] = csum;
}

// ------------------------------------------------------------------------
// k space: SpectralSolver::fft_mean_flow_field (spectral_solver.rs:133-189),
// MagneticSolver::fft_mean_magnetic_field (magnetic_solver.rs:71-95) and both
// update_gradient (spectral_solver.rs:192-229, magnetic_solver.rs:98-135), on
// the half spectrum of the real-to-complex transforms.
//
// The reference applies these operators to the full spectrum of a
// complex-to-complex FFT of each real field and keeps the real part of the
// complex inverse (simulation/mod.rs:399-414).  With X(k) the operator's
// output, Re ifft(X) is the complex-to-real inverse of the Hermitian part
// H(k) = (X(k) + conj X(-k)) / 2, and Im ifft(X) that of
// (X(k) - conj X(-k)) / 2i.  X(-k) is the operator at the mirrored wave
// vector with the spectrum conj sigma(k) (the spectrum of a real field); the
// mirror negates every component of k except a Nyquist one (index n/2 of an
// even n, whose wave number -n/2 is its own mirror).  With no Nyquist index
// the operators give conj X(-k) = X(k) exactly (every operation is odd or
// even in k), so H = X and the anti-Hermitian part is zero: only bins on a
// Nyquist plane evaluate the operators twice.
//
// fwd: [0..9) sigma_k, [9..12) P_k.  out: [0..9) G_k = i k_a u_b, [9..12) u_k,
// [12..21) grad B_k, [21..24) B_k, all [comp][half bin].  Complex products
// with k (imaginary part zero) reduce exactly to real scalings.
// ------------------------------------------------------------------------
__device__ __forceinline__ void flow_ops(const double k[3], const double kn[3], double fac, const double2 *sig,
                                         double2 *o) {
    double2 sg[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        const double2 a0 = sig[3 * r + 0], a1 = sig[3 * r + 1], a2 = sig[3 * r + 2];
        sg[r].x = (a0.x * k[0] + a1.x * k[1]) + a2.x * k[2];
        sg[r].y = (a0.y * k[0] + a1.y * k[1]) + a2.y * k[2];
    }
    const double ksr = (kn[0] * sg[0].x + kn[1] * sg[1].x) + kn[2] * sg[2].x;
    const double ksi = (kn[0] * sg[0].y + kn[1] * sg[1].y) + kn[2] * sg[2].y;
    double2 u[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        const double tr = (sg[r].x - kn[r] * ksr) * fac;
        const double ti = (sg[r].y - kn[r] * ksi) * fac;
        u[r] = make_double2(-ti, tr);  // times i
        o[9 + r] = u[r];
    }
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) o[3 * a + b] = make_double2(-(k[a] * u[b].y), k[a] * u[b].x);
}

__device__ __forceinline__ void mag_ops(const double k[3], const double kn[3], double norm, const double2 *p,
                                        double2 *o) {
    const double dr = (kn[0] * p[0].x + kn[1] * p[1].x) + kn[2] * p[2].x;
    const double di = (kn[0] * p[0].y + kn[1] * p[1].y) + kn[2] * p[2].y;
    double2 b[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        b[r] = make_double2((p[r].x - kn[r] * dr) / norm, (p[r].y - kn[r] * di) / norm);
        o[9 + r] = b[r];
    }
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int bb = 0; bb < 3; ++bb) o[3 * a + bb] = make_double2(-(k[a] * b[bb].y), k[a] * b[bb].x);
}

// ANTI: the anti-Hermitian part (the imaginary parts of the reference's
// complex fields) instead of the Hermitian one
template <bool FLOW, bool MAG, bool ANTI>
__global__ void k_kspace(const double2 *__restrict__ fwd, double2 *__restrict__ out, DevParams P, double screening,
                         double stepx, double stepy, double stepz) {
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    const int nh = P.nhalf;
    if (h >= nh) return;
    const int iz = h % P.hdim[2];
    const int iy = (h / P.hdim[2]) % P.hdim[1];
    const int ix = h / (P.hdim[2] * P.hdim[1]);
    const double k[3] = {kval(ix, P.gx, stepx), kval(iy, P.gy, stepy), kval(iz, P.gz, stepz)};
    const bool nyq[3] = {(P.gx & 1) == 0 && 2 * ix == P.gx, (P.gy & 1) == 0 && 2 * iy == P.gy,
                         (P.gz & 1) == 0 && 2 * iz == P.gz};
    const bool mirror = nyq[0] || nyq[1] || nyq[2];
    const bool kzero = (ix | iy | iz) == 0;
    // |k|^2 = ((0 + kx^2) + ky^2) + kz^2 (fft_helper.rs:80-82)
    double s = (k[0] * k[0] + k[1] * k[1]);
    s = s + k[2] * k[2];
    // 1/|k|^2 via num-complex's real/complex division: s / (s*s); 1/|k| for k-hat;
    // both zero at k = 0 (fft_helper.rs:84-85, 96-97)
    const double ik2 = kzero ? 0.0 : s / (s * s);
    const double inrm = kzero ? 0.0 : 1.0 / sqrt(s);
    const double kn[3] = {k[0] * inrm, k[1] * inrm, k[2] * inrm};
    const double km[3] = {nyq[0] ? k[0] : -k[0], nyq[1] ? k[1] : -k[1], nyq[2] ? k[2] : -k[2]};
    const double knm[3] = {km[0] * inrm, km[1] * inrm, km[2] * inrm};
    const double norm = (double)P.ncell;
    auto emit = [&](int c0, const double2 *X, const double2 *Xm) {
#pragma unroll
        for (int j = 0; j < 12; ++j) {
            double2 v;
            if (!mirror) {
                v = ANTI ? make_double2(0.0, 0.0) : X[j];
            } else if (ANTI) {  // (X - conj Xm) / 2i
                v = make_double2((X[j].y + Xm[j].y) * 0.5, -(X[j].x - Xm[j].x) * 0.5);
            } else {  // (X + conj Xm) / 2
                v = make_double2((X[j].x + Xm[j].x) * 0.5, (X[j].y - Xm[j].y) * 0.5);
            }
            out[(long long)(c0 + j) * nh + h] = v;
        }
    };
    if (FLOW) {
        double2 sig[9], X[12], Xm[12];
#pragma unroll
        for (int j = 0; j < 9; ++j) sig[j] = fwd[(long long)j * nh + h];
        const double fac = (ik2 + screening) / norm;
        flow_ops(k, kn, fac, sig, X);
        if (mirror) {
#pragma unroll
            for (int j = 0; j < 9; ++j) sig[j].y = -sig[j].y;
            flow_ops(km, knm, fac, sig, Xm);
        }
        emit(0, X, Xm);
    }
    if (MAG) {
        double2 pol[3], X[12], Xm[12];
#pragma unroll
        for (int j = 0; j < 3; ++j) pol[j] = fwd[(long long)(9 + j) * nh + h];
        mag_ops(k, kn, norm, pol, X);
        if (mirror) {
#pragma unroll
            for (int j = 0; j < 3; ++j) pol[j].y = -pol[j].y;
            mag_ops(km, knm, norm, pol, Xm);
        }
        emit(12, X, Xm);
    }
}

// real <-> complex copies of a one-cell grid (no axis to transform)
__global__ void k_real_to_complex(const double *__restrict__ src, int count, int sstride, double2 *__restrict__ dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) dst[i] = make_double2(src[(long long)i * sstride], 0.0);
}
__global__ void k_complex_to_real(const double2 *__restrict__ src, int count, double *__restrict__ dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) dst[i] = src[i].x;
}
// the reference's complex field [comp][cell] from its real and imaginary parts
__global__ void k_combine_complex(const double *__restrict__ re, const double *__restrict__ im, long long count,
                                  double2 *__restrict__ dst) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < count) dst[i] = make_double2(re[i], im[i]);
}

// ------------------------------------------------------------------------
// per-cell table: W = (G - G^T) * 0.5, E = (G + G^T) * 0.5 on real parts
// (simulation/mod.rs:302-308), Re u, Re B * mdd, Re grad B (:323-339)
// ------------------------------------------------------------------------
// A table entry: a double, or (with the two-float update) the float pair
// (hi, lo) of that double in the same 8 bytes.
__device__ __forceinline__ void put_entry(double *row, int k, double v, bool pairs) {
    if (pairs) {
        const float h = __double2float_rn(v);
        reinterpret_cast<float2 *>(row)[k] = make_float2(h, __double2float_rn(v - (double)h));
    } else {
        row[k] = v;
    }
}

template <bool FLOW, bool MAG>
__global__ void k_table(const double *__restrict__ inv, DevParams P, double *__restrict__ table, int tstride,
                        double *__restrict__ ctab) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int nc = P.ncell;
    if (c >= nc) return;
    double *row = table + (long long)c * tstride;
    // the two-float update (nearest-cell gather) reads the row as float
    // pairs: u, W, E, the diffusion length (k_contract's, converted here)
    // and B, grad B; the flow solve runs every step, so FLOW marks a full row
    const bool pairs = FLOW && P.f32x2 && !P.gather;
    if (FLOW) {
        double g[9], u[3];
#pragma unroll
        for (int j = 0; j < 9; ++j) g[j] = inv[(long long)j * nc + c];
#pragma unroll
        for (int r = 0; r < 3; ++r) u[r] = inv[(long long)(9 + r) * nc + c];
        const double w01 = (g[1] - g[3]) * 0.5, w02 = (g[2] - g[6]) * 0.5, w12 = (g[5] - g[7]) * 0.5;
        const double e00 = (g[0] + g[0]) * 0.5, e01 = (g[1] + g[3]) * 0.5, e02 = (g[2] + g[6]) * 0.5;
        const double e11 = (g[4] + g[4]) * 0.5, e12 = (g[5] + g[7]) * 0.5, e22 = (g[8] + g[8]) * 0.5;
        const double diff = row[T_DIFF];
#pragma unroll
        for (int r = 0; r < 3; ++r) put_entry(row, T_U + r, u[r], pairs);
        put_entry(row, T_W01, w01, pairs);
        put_entry(row, T_W02, w02, pairs);
        put_entry(row, T_W12, w12, pairs);
        put_entry(row, T_E00, e00, pairs);
        put_entry(row, T_E01, e01, pairs);
        put_entry(row, T_E02, e02, pairs);
        put_entry(row, T_E11, e11, pairs);
        put_entry(row, T_E12, e12, pairs);
        put_entry(row, T_E22, e22, pairs);
        if (pairs) put_entry(row, T_DIFF, diff, true);
        if (ctab) {  // the canonical quasi-2-D chain's row (CT_*), pre-multiplied by dt
            const double v[CTAB_STRIDE] = {u[0] * P.dt, u[1] * P.dt, w01 * P.dt, e00 * P.shape_dt,
                                           e01 * P.shape_dt, e11 * P.shape_dt, diff, 0.0};
            double *cr = ctab + (long long)c * CTAB_STRIDE;
            if (P.f32x2) {  // the same row as float pairs (hi, lo) in the same 64 bytes
#pragma unroll
                for (int k = 0; k < CTAB_STRIDE; ++k) put_entry(cr, k, v[k], true);
            } else {
#pragma unroll
                for (int k = 0; k < CTAB_STRIDE; ++k) cr[k] = v[k];
            }
        }
    }
    if (MAG) {
#pragma unroll
        for (int r = 0; r < 3; ++r) put_entry(row, T_B + r, inv[(long long)(21 + r) * nc + c] * P.mdd, pairs);
#pragma unroll
        for (int j = 0; j < 9; ++j) put_entry(row, T_GB + j, inv[(long long)(12 + j) * nc + c], pairs);
    }
}

// The canonical quasi-2-D step with its increments in two-float arithmetic
// (f32x2.cuh): the noise as floats (Philox) or as pairs of the host noise,
// the cell's float-pair table row ct, and the sums with the FP64 state in
// FP64 (h first, then l) before the periodic wrap.  Its kernel variant is
// compiled for 5 blocks of 256 per SM (48 registers, no spills): the chain
// is bound by instruction issue, and 62.5 % occupancy issues 5 % more per
// clock than the 50 % that 58 registers allow.
template <int NOISE>
__device__ __forceinline__ void langevin_canon_f2(const DevParams &P, double &px, double &py, double &pph,
                                                  const float4 *__restrict__ ct, uint32_t pid,
                                                  const double *__restrict__ noise,
                                                  const unsigned long long *__restrict__ d_step) {
    const xf::CanonTerms T = {(P.mask & M_SELF_PROPULSION) != 0u, (P.mask & M_CONVECTION) != 0u,
                              (P.mask & M_TRANS_DIFFUSION) != 0u, (P.mask & M_ROT_DIFFUSION) != 0u,
                              (P.mask & M_EXTERNAL_FIELD) != 0u, (P.mask & M_JEFFREY_VORTICITY) != 0u,
                              (P.mask & M_JEFFREY_STRAIN) != 0u};
    const xf::f2 dt2 = {P.dt2[0], P.dt2[1]}, re2 = {P.reorient2[0], P.reorient2[1]};
    xf::f2 dx, dy, dph;
    if (NOISE == 0) {
        const NoiseF f = philox_noise_f(P.seed, pid, *d_step);
        // unnormalised: sincos_f2 adds the low part to the reduced angle exactly
        const xf::f2 rot = xf::mul_u(xf::f2{P.sigma2[0], P.sigma2[1]}, f.rad);
        xf::canon_increments(pph, ct, f.xi0, f.xi1, f.sa, rot, T, dt2, re2, dx, dy, dph);
    } else {
        const double *r = noise + 5ull * pid;
        double sa, ca;
        sincos(r[3], &sa, &ca);
        xf::canon_increments(pph, ct, xf::split(r[0]), xf::split(r[1]), xf::split(sa), xf::split(r[4]), T, dt2,
                             re2, dx, dy, dph);
    }
    px = modulo_rare((px + xf::to_double(dx.h)) + xf::to_double(dx.l), P.bx);
    py = modulo_rare((py + xf::to_double(dy.h)) + xf::to_double(dy.l), P.by);
    pph = ref_modulo((pph + xf::to_double(dph.h)) + xf::to_double(dph.l), kTwoPi);
}

static_assert(xf::R_U == T_U && xf::R_W01 == T_W01 && xf::R_W02 == T_W02 && xf::R_W12 == T_W12 &&
                  xf::R_E00 == T_E00 && xf::R_E01 == T_E01 && xf::R_E02 == T_E02 && xf::R_E11 == T_E11 &&
                  xf::R_E12 == T_E12 && xf::R_E22 == T_E22 && xf::R_DIFF == T_DIFF && xf::R_B == T_B &&
                  xf::R_GB == T_GB,
              "the float-pair row has the layout of the double table row");

// The full chain (3-D, and quasi-2-D rows off the canonical state) with its
// increments in two-float arithmetic (xf::full_increments) from the cell's
// float-pair row, then the FP64 sums, the periodic wrap and the angle
// ranges of Particle::pbc / ang_pbc: phi mod 2 pi, theta in [0, pi] (the
// range atan2 gives the reference's new theta).  Quasi2d: z = 0 and
// theta = pi/2 afterwards (simulation/mod.rs:365-368).
template <bool Q2D, int NOISE>
__device__ __forceinline__ void langevin_full_f2(const DevParams &P, double &px, double &py, double &pz,
                                                 double &pph, double &pth, const float2 *__restrict__ row,
                                                 uint32_t pid, const double *__restrict__ noise,
                                                 const unsigned long long *__restrict__ d_step) {
    const uint32_t m = P.mask;
    const xf::FullTerms T = {(m & M_SELF_PROPULSION) != 0u, (m & M_CONVECTION) != 0u, (m & M_MDD_FORCE) != 0u,
                             (m & M_EXTERNAL_FIELD) != 0u,  (m & M_MDD_ROTATION) != 0u, (m & M_JEFFREY_VORTICITY) != 0u,
                             (m & M_JEFFREY_STRAIN) != 0u,  (m & M_STEP) != 0u,      (m & M_TRANS_DIFFUSION) != 0u,
                             (m & M_ROT_DIFFUSION) != 0u};
    const xf::f2 dt2 = {P.dt2[0], P.dt2[1]}, re2 = {P.reorient_f2[0], P.reorient_f2[1]};
    const xf::f2 sh2 = {P.shape2[0], P.shape2[1]}, dr2 = {P.drag2[0], P.drag2[1]};
    xf::FullOut o;
    if (NOISE == 0) {
        const NoiseF f = philox_noise_f(P.seed, pid, *d_step);
        const float xi2 = Q2D ? 0.0f : philox_xi2_f(P.seed, pid, *d_step);
        const xf::f2 rot = xf::mul_u(xf::f2{P.sigma2[0], P.sigma2[1]}, f.rad);
        xf::full_increments(pph, pth, row, f.xi0, f.xi1, xi2, f.sa, xf::axis_cos(f.sa, f.ca), rot, T, dt2, re2,
                            sh2, dr2, o);
    } else {
        const double *r = noise + 5ull * pid;
        double sa, ca;
        sincos(r[3], &sa, &ca);
        xf::full_increments(pph, pth, row, xf::split(r[0]), xf::split(r[1]), xf::split(r[2]), xf::split(sa),
                            xf::split(ca), xf::split(r[4]), T, dt2, re2, sh2, dr2, o);
    }
    px = ref_modulo((px + xf::to_double(o.dp[0].h)) + xf::to_double(o.dp[0].l), P.bx);
    py = ref_modulo((py + xf::to_double(o.dp[1].h)) + xf::to_double(o.dp[1].l), P.by);
    double nphi, nth;
    if (!o.direct) {
        nphi = (pph + xf::to_double(o.a.h)) + xf::to_double(o.a.l);
        nth = (pth + xf::to_double(o.b.h)) + xf::to_double(o.b.l);
        // theta in [0, pi], as the reference's pi/2 - atan2(v2, |v_xy|) (compares on the bits:
        // a negative value other than -0.0 -> 0, a positive one above pi (or a NaN) -> pi)
        const unsigned long long bn = dbits(nth);
        if ((bn & kSignBit) && bn != kSignBit) nth = 0.0;
        else if (!(bn & kSignBit) && bn > dbits(kPi)) nth = kPi;
    } else {
        nphi = xf::to_double(o.a.h) + xf::to_double(o.a.l);
        nth = kPiHalf - (xf::to_double(o.b.h) + xf::to_double(o.b.l));
    }
    pph = ref_modulo(nphi, kTwoPi);
    if (Q2D) {
        pz = 0.0;
        pth = kPiHalf;
    } else {
        pz = ref_modulo((pz + xf::to_double(o.dp[2].h)) + xf::to_double(o.dp[2].l), P.bz);
        pth = nth;
    }
}

// ------------------------------------------------------------------------
// particle update: the loop of src/bin/simulation/mod.rs:318-369 fused with
// the next step's binning (histogram_from) so each step reads and writes the
// particle state once.  NOISE: 0 = Philox on device, 1 = host array [N][5]
// indexed by the caller's particle order.  CANON (quasi2d, every particle in
// the canonical state z = 0, theta = pi/2, no magnetic step, nearest-cell
// gather): the chain of langevin_canon, and z and theta are neither read nor
// written.  F2 (with CANON): the same chain's increments in two-float
// arithmetic (f32x2.cuh) from the float-pair table row, added to the FP64
// state in FP64.  Register budgets of the F2 forms (launch bounds): 5 blocks
// of 256 per SM for the canonical chain, 4 for the 3-D chain (64 registers,
// a few words spilled; 2.02 -> 1.94 ms on the 3-D workload against 3
// blocks), 3 for the quasi-2-D general chain.
// ------------------------------------------------------------------------
template <bool Q2D, bool MAG, int NOISE, bool TRI, bool CANON = false, bool F2 = false>
__global__ void __launch_bounds__(256, F2 ? (CANON ? 5 : (Q2D ? 3 : 4)) : 1) k_update(DevParams P, double *__restrict__ x, double *__restrict__ y,
                                                double *__restrict__ z, double *__restrict__ phi,
                                                double *__restrict__ theta, uint32_t *__restrict__ key,
                                                const uint32_t *__restrict__ id, const double *__restrict__ table,
                                                const double *__restrict__ noise,
                                                const unsigned long long *__restrict__ d_step,
                                                uint32_t *__restrict__ counts_next, uint32_t *__restrict__ errflag) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const int ts = CANON ? CTAB_STRIDE : (MAG || TRI) ? TABLE_STRIDE_MAG : TABLE_STRIDE;
    uint32_t cell = key[i];
    uint32_t pid = id[i];
    double px = x[i], py = y[i], pph = phi[i];
    double pz = CANON ? 0.0 : z[i], pth = CANON ? kPiHalf : theta[i];
    TableFields F{table + (long long)cell * ts};
    double trow[TABLE_STRIDE_MAG];
    if (TRI) {
        trilinear_row<MAG>(table, P, px, py, pz, trow);
        F.r = trow;
    }
    if (CANON && F2) {
        langevin_canon_f2<NOISE>(P, px, py, pph, reinterpret_cast<const float4 *>(F.r), pid, noise, d_step);
    } else if (F2) {
        langevin_full_f2<Q2D, NOISE>(P, px, py, pz, pph, pth, reinterpret_cast<const float2 *>(F.r), pid, noise,
                                     d_step);
    } else {
        double xi[3], ca, sa, rot;
        if (NOISE == 0) {
            philox_noise<Q2D>(P.seed, pid, *d_step, P.sigma_rot, xi, ca, sa, rot);
        } else {
            const double *r = noise + 5ull * pid;
            xi[0] = r[0]; xi[1] = r[1]; xi[2] = r[2];
            sincos(r[3], &sa, &ca);
            rot = r[4];
        }
        if (CANON) {
            langevin_canon(px, py, pph, F.r, xi, sa, rot, P.mask, P.dt, P.reorient_dt, P.bx, P.by);
        } else {
            bool have_theta = Q2D && (__double_as_longlong(pth) == __double_as_longlong(kPiHalf));
            langevin<Q2D>(px, py, pz, pph, pth, F, xi, ca, sa, rot, P.mask, P.dt, P.reorient, P.shape, P.drag,
                          P.bx, P.by, P.bz, have_theta, P.cos_half_pi, P.sin_half_pi);
        }
    }
    uint32_t err = 0, ncell;
    unsigned long long bin;
    bin_particle<Q2D>(P, px, py, pz, pph, pth, ncell, bin, err);
    atomicAdd(counts_next + bin, 1u);
    key[i] = ncell;
    x[i] = px; y[i] = py; phi[i] = pph;
    if (!CANON) {
        z[i] = pz;
        theta[i] = pth;
    }
    if (err) atomicOr(errflag, err);
}

__global__ void k_step_inc(unsigned long long *d_step) { *d_step += 1ull; }

// Initial conditions: Particle::create_isotropic / create_homogeneous
// (src/particle.rs:224-295) with Philox draws (counter (i, ~0, ~0, 3..5),
// outside the range the steps use) instead of Pcg64Mcg.  Rows are written in
// the boundary layout [n][5]; the caller then ingests them like ss_init.
template <bool HOMOGENEOUS>
__global__ void k_sample_initial(DevParams P, double kappa, double *__restrict__ aos, uint32_t *__restrict__ errflag) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    uint2 key = make_uint2((uint32_t)P.seed, (uint32_t)(P.seed >> 32));
    uint4 a = philox4x32_10(make_uint4((uint32_t)i, 0xFFFFFFFFu, 0xFFFFFFFFu, 3u), key);
    uint4 b = philox4x32_10(make_uint4((uint32_t)i, 0xFFFFFFFFu, 0xFFFFFFFFu, 4u), key);
    uint4 c = philox4x32_10(make_uint4((uint32_t)i, 0xFFFFFFFFu, 0xFFFFFFFFu, 5u), key);
    double u[5] = {u12(a.x, a.y) - 1.0, u12(a.z, a.w) - 1.0, u12(b.x, b.y) - 1.0, u12(b.z, b.w) - 1.0,
                   u12(c.x, c.y) - 1.0};
    double x = P.bx * u[0], y = P.by * u[1], z = P.bz * u[2], phi = kTwoPi * u[3], theta;
    if (!HOMOGENEOUS) {
        theta = acos(1.0 - 2.0 * u[4]);  // pdf_sin(2 r), particle.rs:340-342
    } else {
        // pdf_homogeneous_fixpoint, particle.rs:347-360
        theta = acos(log(exp(kappa) - 2.0 * u[4] * sinh(kappa)) / kappa);
        if (theta != theta) atomicOr(errflag, ERR_NONFINITE);
    }
    // Particle::new: modulo / ang_pbc, then pbc
    x = ref_modulo(ref_modulo(x, P.bx), P.bx);
    y = ref_modulo(ref_modulo(y, P.by), P.by);
    z = ref_modulo(ref_modulo(z, P.bz), P.bz);
    ref_ang_pbc(phi, theta);
    ref_ang_pbc(phi, theta);
    if (HOMOGENEOUS) {
        // rotate the orientation by -pi/2 about x (place_homogeneous,
        // particle.rs:271-276; Rodrigues with k = (1, 0, 0)), then
        // Orientation::from_vector_mut
        double sp, cp, st, ct;
        sincos(phi, &sp, &cp);
        sincos(theta, &st, &ct);
        double n0 = st * cp, n1 = st * sp, n2 = ct;
        double sr, cr;
        sincos(-kPiHalf, &sr, &cr);
        double r0 = n0;  // the component along the axis is unchanged
        double r1 = n1 * cr - n2 * sr;
        double r2 = n2 * cr + n1 * sr;
        phi = atan2(r1, r0);
        theta = kPiHalf - atan2(r2, sqrt(r0 * r0 + r1 * r1));
    }
    double *p = aos + 5 * i;
    p[0] = x; p[1] = y; p[2] = z; p[3] = phi; p[4] = theta;
}

// the Philox noise of step t for every particle, as RandomVector rows in the
// caller's order
template <bool Q2D>
__global__ void k_noise(DevParams P, unsigned long long t, double *__restrict__ out) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    double xi[3], ca, sa, rot, alpha;
    philox_noise<Q2D, true>(P.seed, (uint32_t)i, t, P.sigma_rot, xi, ca, sa, rot, &alpha);
    double *r = out + 5 * i;
    r[0] = xi[0]; r[1] = xi[1]; r[2] = xi[2]; r[3] = alpha; r[4] = rot;
}

// ------------------------------------------------------------------------
// counting sort by cell
// ------------------------------------------------------------------------
// exclusive scan of cellcount into cursor (one block)
__global__ void __launch_bounds__(1024) k_scan(const uint32_t *__restrict__ cnt, int n, uint32_t *__restrict__ out) {
    __shared__ uint32_t part[1024];
    int t = threadIdx.x;
    int per = (n + 1023) / 1024;
    int lo = t * per, hi = min(n, lo + per);
    uint32_t s = 0;
    for (int i = lo; i < hi; ++i) s += cnt[i];
    part[t] = s;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        uint32_t v = (t >= o) ? part[t - o] : 0u;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    uint32_t run = part[t] - s;
    for (int i = lo; i < hi; ++i) {
        uint32_t c = cnt[i];
        out[i] = run;
        run += c;
    }
}

// scatter slot i to cursor[key] + rank; ranks handed out with one atomic per
// group of lanes sharing a cell (warp-aggregated)
__global__ void __launch_bounds__(256) k_scatter(unsigned long long n, const double *__restrict__ x,
                                                 const double *__restrict__ y, const double *__restrict__ z,
                                                 const double *__restrict__ phi, const double *__restrict__ theta,
                                                 const uint32_t *__restrict__ key, const uint32_t *__restrict__ id,
                                                 double *__restrict__ x2, double *__restrict__ y2,
                                                 double *__restrict__ z2, double *__restrict__ phi2,
                                                 double *__restrict__ theta2, uint32_t *__restrict__ key2,
                                                 uint32_t *__restrict__ id2, uint32_t *__restrict__ cursor) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    int lane = threadIdx.x & 31;
    uint32_t k = key[i];
    unsigned act = __activemask();
    unsigned same = __match_any_sync(act, k);
    int leader = __ffs(same) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(cursor + k, (uint32_t)__popc(same));
    base = __shfl_sync(same, base, leader);
    uint32_t dst = base + (uint32_t)__popc(same & ((1u << lane) - 1u));
    x2[dst] = x[i]; y2[dst] = y[i]; z2[dst] = z[i]; phi2[dst] = phi[i]; theta2[dst] = theta[i];
    key2[dst] = k; id2[dst] = id[i];
}

// ------------------------------------------------------------------------
// misc
// ------------------------------------------------------------------------
__global__ void k_zero_u32(uint32_t *__restrict__ p, long long n) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    long long stride = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += stride) p[i] = 0u;
}

__global__ void k_real_parts(const double2 *__restrict__ src, long long count, double *__restrict__ dst) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= count) return;
    dst[i] = src[i].x;
}

__global__ void k_half_pi(double *out) {
    double s, c;
    sincos(kPiHalf, &s, &c);
    out[0] = c;
    out[1] = s;
}

// the Langevin chain on independent particles with shared arguments
template <bool Q2D>
__global__ void k_langevin_args(const double *__restrict__ in, unsigned long long n, uint32_t mask,
                                const double *__restrict__ a /* ss_langevin_args as doubles */,
                                double *__restrict__ out) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    // field offsets inside ss_langevin_args (all doubles)
    const double *flow = a + 0, *gradb = a + 4, *b = a + 14, *vort = a + 17, *strain = a + 27;
    double drag = a[3], reorient = a[13], shape = a[26], dt = a[36], diff = a[40];
    const double *xi = a + 37;
    double alpha = a[41], rot = a[42], bx = a[43], by = a[44], bz = a[45];
    MatrixFields F{flow, gradb, b, vort, strain, diff};
    double px = in[5 * i], py = in[5 * i + 1], pz = in[5 * i + 2], pph = in[5 * i + 3], pth = in[5 * i + 4];
    double sa, ca, xv[3] = {xi[0], xi[1], xi[2]};
    sincos(alpha, &sa, &ca);
    langevin<false>(px, py, pz, pph, pth, F, xv, ca, sa, rot, mask, dt, reorient, shape, drag, bx, by, bz, false,
                    0.0, 0.0);
    out[5 * i] = px; out[5 * i + 1] = py; out[5 * i + 2] = pz; out[5 * i + 3] = pph; out[5 * i + 4] = pth;
}

// FP64 FMA throughput probe: every thread runs 8 independent FMA chains of
// `iters` steps (x <- x a + b with |a| < 1, so the chains stay finite); the
// sum is written so that the chains are not removed.
__global__ void __launch_bounds__(256) k_fp64_rate(int iters, double a, double b, double *__restrict__ out) {
    double x[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = (double)(threadIdx.x + k);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
    }
    double sum = 0.0;
#pragma unroll
    for (int k = 0; k < 8; ++k) sum += x[k];
    out[blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x] = sum;
}

// ========================================================================
// launch wrappers
// ========================================================================
static inline unsigned nblocks(unsigned long long n, unsigned bs) { return (unsigned)((n + bs - 1) / bs); }

void launch_scan_rows(cudaStream_t s, const double *aos, unsigned long long n, unsigned long long *scan) {
    if (n) k_scan_rows<<<nblocks(n, 256), 256, 0, s>>>(aos, n, scan);
}

void launch_egest(cudaStream_t s, unsigned long long n, double *const xs[5], const uint32_t *id, double *aos) {
    if (!n) return;
    k_egest<<<nblocks(n, 256), 256, 0, s>>>(n, xs[0], xs[1], xs[2], xs[3], xs[4], id, aos);
}

void launch_sort_rows(cudaStream_t s, const double *aos, unsigned long long n, const DevParams &P,
                      uint32_t *cellkey, uint32_t *cellcount, uint32_t *cursor, double *sorted, uint32_t *orig) {
    if (!n) return;
    launch_zero_u32(s, cellcount, P.ncell);
    k_row_cells<<<nblocks(n, 256), 256, 0, s>>>(aos, n, P, cellkey, cellcount);
    launch_scan(s, cellcount, P.ncell, cursor);
    k_sort_rows<<<nblocks(n, 256), 256, 0, s>>>(aos, n, cellkey, cursor, sorted, orig);
}

void launch_ingest_bin(cudaStream_t s, bool canon, const double *aos, unsigned long long n, const DevParams &P,
                       double *const xs[5], uint32_t *id, uint32_t *key, uint32_t *counts, uint32_t *err) {
    if (!n) return;
    if (canon)
        k_ingest_bin<true><<<nblocks(n, 256), 256, 0, s>>>(aos, n, P, xs[0], xs[1], xs[2], xs[3], xs[4], id, key,
                                                           counts, err);
    else
        k_ingest_bin<false><<<nblocks(n, 256), 256, 0, s>>>(aos, n, P, xs[0], xs[1], xs[2], xs[3], xs[4], id, key,
                                                            counts, err);
}

void launch_ingest_bin_check(cudaStream_t s, const double *aos, unsigned long long n, unsigned long long off,
                             const DevParams &P, double *const xs[5], uint32_t *id, uint32_t *key,
                             uint32_t *counts, unsigned long long *scan, uint32_t *err) {
    if (!n) return;
    k_ingest_bin_check<<<nblocks(n, 256), 256, 0, s>>>(aos, n, off, P, xs[0], xs[1], xs[2], xs[3], xs[4], id, key,
                                                       counts, scan, err);
}

void launch_counts_to_dist(cudaStream_t s, const uint32_t *counts, const DevParams &P, double *dist) {
    k_counts_to_dist<<<nblocks(P.nbins, 256), 256, 0, s>>>(counts, P.nbins, P, dist);
}

void launch_contract(cudaStream_t s, bool stress, bool mag, const uint32_t *counts, const double *dist,
                     const double *lut, int lut_n, const double *kern, const DevParams &P, double *fwd,
                     double *table, int tstride, uint32_t *cellcount) {
    unsigned blocks = nblocks((unsigned long long)P.ncell, 64);
    const size_t smem = 12ull * P.nang * sizeof(double);
    const bool use_smem = smem <= 48 * 1024;
    const size_t sm = use_smem ? smem : 0;
#define SS_CONTRACT(S, M, D)                                                                                     \
    do {                                                                                                         \
        if (use_smem)                                                                                            \
            k_contract<S, M, D, true><<<blocks, 64, sm, s>>>(counts, dist, lut, lut_n, kern, P, fwd, table,     \
                                                             tstride, cellcount);                                \
        else                                                                                                     \
            k_contract<S, M, D, false><<<blocks, 64, 0, s>>>(counts, dist, lut, lut_n, kern, P, fwd, table,     \
                                                             tstride, cellcount);                                \
    } while (0)
    bool fd = dist != nullptr;
    if (stress && mag) { if (fd) SS_CONTRACT(true, true, true); else SS_CONTRACT(true, true, false); }
    else if (stress) { if (fd) SS_CONTRACT(true, false, true); else SS_CONTRACT(true, false, false); }
    else { if (fd) SS_CONTRACT(false, true, true); else SS_CONTRACT(false, true, false); }
#undef SS_CONTRACT
}

void launch_kspace(cudaStream_t s, bool flow, bool mag, bool anti, const double2 *fwd, double2 *inv,
                   const DevParams &P, double screening) {
    double sx = kTwoPi / P.bx, sy = kTwoPi / P.by, sz = kTwoPi / P.bz;
    unsigned b = nblocks(P.nhalf, 128);
#define SS_KS(F, M)                                                                   \
    do {                                                                              \
        if (anti) k_kspace<F, M, true><<<b, 128, 0, s>>>(fwd, inv, P, screening, sx, sy, sz); \
        else k_kspace<F, M, false><<<b, 128, 0, s>>>(fwd, inv, P, screening, sx, sy, sz);     \
    } while (0)
    if (flow && mag) SS_KS(true, true);
    else if (flow) SS_KS(true, false);
    else SS_KS(false, true);
#undef SS_KS
}

void launch_real_to_complex(cudaStream_t s, const double *src, int count, int sstride, double2 *dst) {
    if (count > 0) k_real_to_complex<<<nblocks(count, 128), 128, 0, s>>>(src, count, sstride, dst);
}
void launch_complex_to_real(cudaStream_t s, const double2 *src, int count, double *dst) {
    if (count > 0) k_complex_to_real<<<nblocks(count, 128), 128, 0, s>>>(src, count, dst);
}
void launch_combine_complex(cudaStream_t s, const double *re, const double *im, long long count, double2 *dst) {
    if (count > 0) k_combine_complex<<<nblocks(count, 256), 256, 0, s>>>(re, im, count, dst);
}

void launch_table(cudaStream_t s, bool flow, bool mag, const double *inv, const DevParams &P, double *table,
                  int tstride, double *ctab) {
    unsigned b = nblocks(P.ncell, 128);
    if (flow && mag) k_table<true, true><<<b, 128, 0, s>>>(inv, P, table, tstride, ctab);
    else if (flow) k_table<true, false><<<b, 128, 0, s>>>(inv, P, table, tstride, ctab);
    else k_table<false, true><<<b, 128, 0, s>>>(inv, P, table, tstride, nullptr);
}

void launch_update(cudaStream_t s, bool q2d, bool canon, bool mag, bool host_noise, const DevParams &P,
                   double *const xs[5], uint32_t *key, const uint32_t *id, const double *table, const double *ctab,
                   const double *noise, const unsigned long long *d_step, uint32_t *counts_next, uint32_t *err) {
    if (!P.n) return;
    unsigned b = nblocks(P.n, 256);
    if (q2d && canon && ctab && !mag && !P.gather && !(P.mask & (M_MDD_FORCE | M_MDD_ROTATION))) {
#define SS_CANON(N, F)                                                                                      \
    k_update<true, false, N, false, true, F><<<b, 256, 0, s>>>(P, xs[0], xs[1], xs[2], xs[3], xs[4], key, id, \
                                                               ctab, noise, d_step, counts_next, err)
        if (P.f32x2) { if (host_noise) SS_CANON(1, true); else SS_CANON(0, true); }
        else { if (host_noise) SS_CANON(1, false); else SS_CANON(0, false); }
#undef SS_CANON
        return;
    }
#define SS_UPD(Q, M, N, T)                                                                                   \
    k_update<Q, M, N, T><<<b, 256, 0, s>>>(P, xs[0], xs[1], xs[2], xs[3], xs[4], key, id, table, noise, d_step, \
                                           counts_next, err)
#define SS_UPD_F2(Q, M, N)                                                                                  \
    k_update<Q, M, N, false, false, true><<<b, 256, 0, s>>>(P, xs[0], xs[1], xs[2], xs[3], xs[4], key, id, table, \
                                                            noise, d_step, counts_next, err)
    // with the two-float mode (nearest-cell gather) every update reads the
    // float-pair rows k_table wrote
#define SS_UPD_T(Q, M, N)                   \
    do {                                    \
        if (P.gather) SS_UPD(Q, M, N, true); \
        else if (P.f32x2) SS_UPD_F2(Q, M, N); \
        else SS_UPD(Q, M, N, false);        \
    } while (0)
    if (q2d) {
        if (mag) { if (host_noise) SS_UPD_T(true, true, 1); else SS_UPD_T(true, true, 0); }
        else { if (host_noise) SS_UPD_T(true, false, 1); else SS_UPD_T(true, false, 0); }
    } else {
        if (mag) { if (host_noise) SS_UPD_T(false, true, 1); else SS_UPD_T(false, true, 0); }
        else { if (host_noise) SS_UPD_T(false, false, 1); else SS_UPD_T(false, false, 0); }
    }
#undef SS_UPD_T
#undef SS_UPD_F2
#undef SS_UPD
}

void launch_step_inc(cudaStream_t s, unsigned long long *d_step) { k_step_inc<<<1, 1, 0, s>>>(d_step); }

void launch_sample_initial(cudaStream_t s, bool homogeneous, const DevParams &P, double kappa, double *aos,
                           uint32_t *err) {
    if (!P.n) return;
    if (homogeneous) k_sample_initial<true><<<nblocks(P.n, 256), 256, 0, s>>>(P, kappa, aos, err);
    else k_sample_initial<false><<<nblocks(P.n, 256), 256, 0, s>>>(P, kappa, aos, err);
}

void launch_noise(cudaStream_t s, bool q2d, const DevParams &P, unsigned long long t, double *out) {
    if (!P.n) return;
    if (q2d) k_noise<true><<<nblocks(P.n, 256), 256, 0, s>>>(P, t, out);
    else k_noise<false><<<nblocks(P.n, 256), 256, 0, s>>>(P, t, out);
}

void launch_scan(cudaStream_t s, const uint32_t *cnt, int n, uint32_t *out) { k_scan<<<1, 1024, 0, s>>>(cnt, n, out); }

void launch_scatter(cudaStream_t s, unsigned long long n, double *const src[5], const uint32_t *key,
                    const uint32_t *id, double *const dst[5], uint32_t *key2, uint32_t *id2, uint32_t *cursor) {
    if (!n) return;
    k_scatter<<<nblocks(n, 256), 256, 0, s>>>(n, src[0], src[1], src[2], src[3], src[4], key, id, dst[0], dst[1],
                                              dst[2], dst[3], dst[4], key2, id2, cursor);
}

void launch_zero_u32(cudaStream_t s, uint32_t *p, long long n) {
    if (n <= 0) return;
    long long b = (n + 255) / 256;
    if (b > 152 * 64) b = 152 * 64;
    k_zero_u32<<<(unsigned)b, 256, 0, s>>>(p, n);
}

void launch_real_parts(cudaStream_t s, const double2 *src, long long count, double *dst) {
    if (count <= 0) return;
    k_real_parts<<<nblocks(count, 256), 256, 0, s>>>(src, count, dst);
}

void launch_half_pi(cudaStream_t s, double *out) { k_half_pi<<<1, 1, 0, s>>>(out); }

void launch_langevin_args(cudaStream_t s, const double *in, unsigned long long n, uint32_t mask, const double *args,
                          double *out) {
    if (!n) return;
    k_langevin_args<false><<<nblocks(n, 128), 128, 0, s>>>(in, n, mask, args, out);
}

void launch_fp64_rate(cudaStream_t s, unsigned blocks, int iters, double *out) {
    k_fp64_rate<<<blocks, 256, 0, s>>>(iters, 0.999999, 1e-3, out);
}

}  // namespace ss
