/*
 * ss_oracle.c -- CPU FP64 restatement of the stochasticsampling timestep.
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT: the parity checker and the timed CPU
 * reference leg of the benchmark.  See ss_oracle.h for the scope and for the
 * third-party algorithms restated here.  Must be compiled with
 * -ffp-contract=off so that no multiply-add is fused: the reference (Rust,
 * LLVM defaults) never fuses either, and the results must not depend on
 * whether the host CPU has FMA.
 *
 * Parallel structure mirrors the reference: histogram and stress
 * contraction serial, FFT components / k-space loops / particle loop
 * parallel (OpenMP here, rayon there).
 */
#include "ss_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* std::f64::consts::PI, src/consts.rs:8 (TWOPI = 2*PI), src/particle.rs:24 */
static const double PI = 3.14159265358979323846;
#define TWOPI (2.0 * PI)
#define PIHALF (PI / 2.0)

/* ===================================================================== */
/* particle.rs                                                           */
/* ===================================================================== */

/* src/particle.rs:26-35 ; Rust `%` on f64 is C fmod */
double orc_modulo(double f, double m) {
    double r = fmod(f, m);
    if (r < 0.0) return r + fabs(m);
    return r;
}

/* src/particle.rs:37-44 */
void orc_ang_pbc(double phi, double theta, double out[2]) {
    theta = orc_modulo(theta, TWOPI);
    if (theta > PI) {
        out[0] = orc_modulo(phi + PI, TWOPI);
        out[1] = TWOPI - theta;
    } else {
        out[0] = orc_modulo(phi, TWOPI);
        out[1] = theta;
    }
}

static void particle_pbc(const orc_settings *s, double p[5]) {
    /* src/particle.rs:72-76, 123-127, 219-222 */
    double o[2];
    p[0] = orc_modulo(p[0], s->bx);
    p[1] = orc_modulo(p[1], s->by);
    p[2] = orc_modulo(p[2], s->bz);
    orc_ang_pbc(p[3], p[4], o);
    p[3] = o[0];
    p[4] = o[1];
}

/* Particle::new, src/particle.rs:186-201: Position::new + Orientation::new, then pbc */
void orc_particle_new(const orc_settings *s, const double in[5], double out[5]) {
    double o[2];
    out[0] = orc_modulo(in[0], s->bx);
    out[1] = orc_modulo(in[1], s->by);
    out[2] = orc_modulo(in[2], s->bz);
    orc_ang_pbc(in[3], in[4], o);
    out[3] = o[0];
    out[4] = o[1];
    particle_pbc(s, out);
}

/* Orientation::from_vector, src/particle.rs:106-121 */
void orc_from_vector(const double v[3], double out[2]) {
    double rxy = sqrt(v[0] * v[0] + v[1] * v[1]);
    out[0] = atan2(v[1], v[0]);
    out[1] = PIHALF - atan2(v[2], rxy);
}

/* ===================================================================== */
/* mesh / distribution                                                   */
/* ===================================================================== */

/* GridWidth::new, src/mesh/grid_width.rs:23-31 */
void orc_grid_width(const orc_settings *s, double gw[5]) {
    gw[0] = s->bx / (double)s->gx;
    gw[1] = s->by / (double)s->gy;
    gw[2] = s->bz / (double)s->gz;
    gw[3] = TWOPI / (double)s->gphi;
    gw[4] = PI / (double)s->gtheta;
}

/* Rust `f64 as usize`: saturating, NaN -> 0 */
static uint64_t as_usize(double v) {
    if (!(v >= 0.0)) return 0;
    if (v >= 18446744073709551615.0) return UINT64_MAX;
    return (uint64_t)v;
}

/* Distribution::coord_to_grid, src/distribution/mod.rs:86-141 */
void orc_coord_to_grid(const orc_settings *s, const double p[5], uint64_t g[5]) {
    double gw[5];
    orc_grid_width(s, gw);
    g[0] = as_usize(floor(p[0] / gw[0]));
    g[1] = as_usize(floor(p[1] / gw[1]));
    g[2] = as_usize(floor(p[2] / gw[2]));
    g[3] = as_usize(floor(p[3] / gw[3]));
    g[4] = as_usize(floor(p[4] / gw[4]));
    if (g[0] == s->gx) g[0] -= 1;
    if (g[1] == s->gy) g[1] -= 1;
    if (g[2] == s->gz) g[2] -= 1;
    if (g[3] == s->gphi) g[3] -= 1;
    if (g[4] == s->gtheta) g[4] -= 1;
}

/* get_cell_index, src/mesh/mod.rs:44-66 */
void orc_cell_index(const orc_settings *s, const double p[5], uint64_t g[3]) {
    double gw[5];
    orc_grid_width(s, gw);
    g[0] = as_usize(floor(p[0] / gw[0]));
    g[1] = as_usize(floor(p[1] / gw[1]));
    g[2] = as_usize(floor(p[2] / gw[2]));
    if (g[0] == s->gx) g[0] -= 1;
    if (g[1] == s->gy) g[1] -= 1;
    if (g[2] == s->gz) g[2] -= 1;
}

/* get_k_sampling, src/mesh/fft_helper.rs:26-51: FFTW order, Nyquist negative */
void orc_k_sampling(uint64_t n, double box, double *out) {
    int64_t a = (int64_t)(n / 2);
    int64_t b = (int64_t)((n % 2 == 0) ? n / 2 : n / 2 + 1);
    double step = TWOPI / box;
    for (int64_t i = 0; i < b; ++i) out[i] = (double)i * step;            /* values[a..] */
    for (int64_t i = 0; i < a; ++i) out[b + i] = (double)(i - a) * step;  /* values[..a] */
}

static void k_axes(const orc_settings *s, double **kx, double **ky, double **kz) {
    *kx = (double *)malloc(sizeof(double) * s->gx);
    *ky = (double *)malloc(sizeof(double) * s->gy);
    *kz = (double *)malloc(sizeof(double) * s->gz);
    orc_k_sampling(s->gx, s->bx, *kx);
    orc_k_sampling(s->gy, s->by, *ky);
    orc_k_sampling(s->gz, s->bz, *kz);
}

/* get_k_mesh, src/mesh/fft_helper.rs:57-60 + mesh3d src/mesh/mod.rs:10-42 */
void orc_k_mesh(const orc_settings *s, double *out) {
    double *kx, *ky, *kz;
    uint64_t n = s->gx * s->gy * s->gz, c = 0;
    k_axes(s, &kx, &ky, &kz);
    for (uint64_t i = 0; i < s->gx; ++i)
        for (uint64_t j = 0; j < s->gy; ++j)
            for (uint64_t l = 0; l < s->gz; ++l, ++c) {
                out[c] = kx[i];
                out[n + c] = ky[j];
                out[2 * n + c] = kz[l];
            }
    free(kx); free(ky); free(kz);
}

/* |k|^2 as ndarray computes it: (k*k) per component, then sum_axis(0)
 * sequentially from zero, src/mesh/fft_helper.rs:80-82 */
static double k_norm_sq(double kx, double ky, double kz) {
    double s = 0.0;
    s = s + kx * kx;
    s = s + ky * ky;
    s = s + kz * kz;
    return s;
}

/* get_inverse_norm_squared, src/mesh/fft_helper.rs:79-88.  `1. / v` for a
 * Complex v goes through num-complex 0.2.3's real/complex division:
 * (1*re)/(re*re + im*im) with im = 0. */
static double inv_norm_sq(double s) { return (1.0 * s) / (s * s + 0.0 * 0.0); }
/* get_inverse_norm, src/mesh/fft_helper.rs:91-99 */
static double inv_norm(double s) { return 1.0 / sqrt(s); }

void orc_inverse_norm_squared(const orc_settings *s, double *out) {
    double *kx, *ky, *kz;
    uint64_t c = 0;
    k_axes(s, &kx, &ky, &kz);
    for (uint64_t i = 0; i < s->gx; ++i)
        for (uint64_t j = 0; j < s->gy; ++j)
            for (uint64_t l = 0; l < s->gz; ++l, ++c)
                out[c] = inv_norm_sq(k_norm_sq(kx[i], ky[j], kz[l]));
    out[0] = 0.0;
    free(kx); free(ky); free(kz);
}

/* get_norm_k_mesh, src/mesh/fft_helper.rs:67-74 */
void orc_norm_k_mesh(const orc_settings *s, double *out) {
    double *kx, *ky, *kz;
    uint64_t n = s->gx * s->gy * s->gz, c = 0;
    k_axes(s, &kx, &ky, &kz);
    for (uint64_t i = 0; i < s->gx; ++i)
        for (uint64_t j = 0; j < s->gy; ++j)
            for (uint64_t l = 0; l < s->gz; ++l, ++c) {
                double inv = (c == 0) ? 0.0 : inv_norm(k_norm_sq(kx[i], ky[j], kz[l]));
                out[c] = kx[i] * inv;
                out[n + c] = ky[j] * inv;
                out[2 * n + c] = kz[l] * inv;
            }
    free(kx); free(ky); free(kz);
}

/* Distribution::histogram_from, src/distribution/mod.rs:146-160 (serial) */
void orc_histogram(const orc_settings *s, const double *particles, uint64_t n, double *dist) {
    uint64_t nb = s->gx * s->gy * s->gz * s->gphi * s->gtheta;
    memset(dist, 0, sizeof(double) * nb);
    for (uint64_t i = 0; i < n; ++i) {
        uint64_t g[5];
        orc_coord_to_grid(s, particles + 5 * i, g);
        uint64_t idx = (((g[0] * s->gy + g[1]) * s->gz + g[2]) * s->gphi + g[3]) * s->gtheta + g[4];
        dist[idx] += 1.0;
    }
}

/* Distribution::sample_from, src/distribution/mod.rs:164-184 */
void orc_sample_from(const orc_settings *s, const double *particles, uint64_t n, double *dist) {
    double gw[5];
    uint64_t nb = s->gx * s->gy * s->gz * s->gphi * s->gtheta;
    orc_histogram(s, particles, n, dist);
    orc_grid_width(s, gw);
    double d = gw[0] * gw[1] * gw[2] * gw[3] * gw[4] * (double)n;
    for (uint64_t i = 0; i < nb; ++i) dist[i] /= d;
}

/* ===================================================================== */
/* angle kernels                                                         */
/* ===================================================================== */

/* ndarray 0.12.1 Array::linspace(start, end, n): start + step * i with
 * step = (end - start) / (n - 1), step = 0 for n <= 1 */
static double linspace_at(double start, double end, uint64_t n, uint64_t i) {
    double step = (n > 1) ? (end - start) / ((double)n - 1.0) : 0.0;
    return start + step * (double)i;
}

/* stresses::stress_active, src/flowfield/stress.rs:103-119 */
void orc_stress_active(double phi, double theta, double s[9]) {
    double cp = cos(phi), sp = sin(phi), ct = cos(theta), st = sin(theta);
    s[0] = -(1. / 3.) + cp * cp * st * st;
    s[1] = cp * st * st * sp;
    s[2] = ct * cp * st;
    s[3] = cp * st * st * sp;
    s[4] = -(1. / 3.) + st * st * sp * sp;
    s[5] = ct * st * sp;
    s[6] = ct * cp * st;
    s[7] = ct * st * sp;
    s[8] = -(1. / 3.) + ct * ct;
}

/* stresses::stress_magnetic, src/flowfield/stress.rs:125-141 */
void orc_stress_magnetic(double phi, double theta, double s[9]) {
    double cp = cos(phi), ct = cos(theta), st = sin(theta);
    s[0] = 0.;
    s[1] = cp * st;
    s[2] = 0.;
    s[3] = -cp * st;
    s[4] = 0.;
    s[5] = -ct;
    s[6] = 0.;
    s[7] = ct;
    s[8] = 0.;
    for (int i = 0; i < 9; ++i) s[i] = s[i] * 0.5;
}

/* stresses::stress_magnetic_rods, src/flowfield/stress.rs:144-159 (powi(2) = x*x) */
void orc_stress_magnetic_rods(double phi, double theta, double s[9]) {
    double cp = cos(phi), sp = sin(phi), ct = cos(theta), st = sin(theta);
    double c2p = cos(2. * phi), c2t = cos(2. * theta), s2t = sin(2. * theta);
    s[0] = 2. * ct * (cp * cp) * (st * st);
    s[1] = ct * (st * st) * c2p;
    s[2] = c2t * cp * st;
    s[3] = ct * (st * st) * c2p;
    s[4] = st * s2t * (sp * sp);
    s[5] = c2t * st * sp;
    s[6] = c2t * cp * st;
    s[7] = c2t * st * sp;
    s[8] = -2. * ct * (st * st);
    for (int i = 0; i < 9; ++i) s[i] = s[i] * 0.5;
}

/* stress_kernel, src/flowfield/stress.rs:29-56, with the closure of
 * src/bin/simulation/mod.rs:100-104 (active*Sa + magnetic*Sm + shape*Sr) */
void orc_stress_kernel(const orc_settings *s, double *out) {
    double gw[5];
    orc_grid_width(s, gw);
    double hp = gw[3] / 2., ht = gw[4] / 2.;
    uint64_t na = s->gphi * s->gtheta;
    for (uint64_t i = 0; i < s->gphi; ++i) {
        double phi = linspace_at(0. + hp, TWOPI - hp, s->gphi, i);
        for (uint64_t j = 0; j < s->gtheta; ++j) {
            double theta = linspace_at(0. + ht, PI - ht, s->gtheta, j);
            double a[9], m[9], r[9];
            orc_stress_active(phi, theta, a);
            orc_stress_magnetic(phi, theta, m);
            orc_stress_magnetic_rods(phi, theta, r);
            for (int c = 0; c < 9; ++c)
                out[(uint64_t)c * na + i * s->gtheta + j] =
                    s->stress_active * a[c] + s->stress_magnetic * m[c] + s->shape * r[c];
        }
    }
}

/* orientation_kernel, src/polarization/director.rs:69-92 (Orientation::new
 * applies ang_pbc, then to_vector) */
void orc_orientation_kernel(const orc_settings *s, double *out) {
    double gw[5];
    orc_grid_width(s, gw);
    double hp = gw[3] / 2., ht = gw[4] / 2.;
    uint64_t na = s->gphi * s->gtheta;
    for (uint64_t i = 0; i < s->gphi; ++i) {
        double phi = linspace_at(0. + hp, TWOPI - hp, s->gphi, i);
        for (uint64_t j = 0; j < s->gtheta; ++j) {
            double theta = linspace_at(0. + ht, PI - ht, s->gtheta, j);
            double o[2];
            orc_ang_pbc(phi, theta, o);
            double cp = cos(o[0]), sp = sin(o[0]), ct = cos(o[1]), st = sin(o[1]);
            out[0 * na + i * s->gtheta + j] = st * cp;
            out[1 * na + i * s->gtheta + j] = st * sp;
            out[2 * na + i * s->gtheta + j] = ct;
        }
    }
}

/* ndarray 0.12.1 unrolled_dot (numeric_util.rs): eight partial sums over
 * blocks of eight, combined pairwise (p0+p4), (p1+p5), (p2+p6), (p3+p7) into
 * the running sum, then the tail added in order. */
static double unrolled_dot(const double *x, const double *y, uint64_t n) {
    double sum = 0.0;
    double p0 = 0, p1 = 0, p2 = 0, p3 = 0, p4 = 0, p5 = 0, p6 = 0, p7 = 0;
    uint64_t i = 0;
    for (; i + 8 <= n; i += 8) {
        p0 = p0 + x[i + 0] * y[i + 0];
        p1 = p1 + x[i + 1] * y[i + 1];
        p2 = p2 + x[i + 2] * y[i + 2];
        p3 = p3 + x[i + 3] * y[i + 3];
        p4 = p4 + x[i + 4] * y[i + 4];
        p5 = p5 + x[i + 5] * y[i + 5];
        p6 = p6 + x[i + 6] * y[i + 6];
        p7 = p7 + x[i + 7] * y[i + 7];
    }
    sum = sum + (p0 + p4);
    sum = sum + (p1 + p5);
    sum = sum + (p2 + p6);
    sum = sum + (p3 + p7);
    for (; i < n; ++i) sum = sum + x[i] * y[i];
    return sum;
}

/* average_stress, src/flowfield/stress.rs:60-96 (serial double loop) */
void orc_average_stress(const orc_settings *s, const double *kernel, const double *dist,
                        double *stress) {
    double gw[5];
    orc_grid_width(s, gw);
    uint64_t na = s->gphi * s->gtheta, nc = s->gx * s->gy * s->gz;
    double measure = gw[3] * gw[4];
    for (uint64_t ij = 0; ij < 9; ++ij)
        for (uint64_t c = 0; c < nc; ++c) {
            stress[2 * (ij * nc + c)] = unrolled_dot(kernel + ij * na, dist + c * na, na) * measure;
            stress[2 * (ij * nc + c) + 1] = 0.0;
        }
}

/* DirectorField::from_distribution, src/polarization/director.rs:36-61 */
void orc_director_field(const orc_settings *s, const double *dist, double *p) {
    double gw[5];
    orc_grid_width(s, gw);
    uint64_t na = s->gphi * s->gtheta, nc = s->gx * s->gy * s->gz;
    double *kern = (double *)malloc(sizeof(double) * 3 * na);
    orc_orientation_kernel(s, kern);
    double measure = gw[3] * gw[4];
    for (uint64_t c = 0; c < nc; ++c)
        for (uint64_t i = 0; i < 3; ++i) {
            p[2 * (i * nc + c)] = unrolled_dot(kern + i * na, dist + c * na, na) * measure;
            p[2 * (i * nc + c) + 1] = 0.0;
        }
    free(kern);
}

/* ===================================================================== */
/* FFT: unnormalised complex DFT, X_k = sum_j x_j exp(sign*2*pi*i*j*k/n), */
/* recursive mixed radix (smallest prime factor first, direct DFT for a   */
/* prime length).  Stands in for FFTW's c2c plans                         */
/* (crates/fftw3/src/fft.rs:156-178, 226-231).                           */
/* ===================================================================== */

typedef struct { double re, im; } cplx;

static uint64_t smallest_factor(uint64_t n) {
    if (n % 2 == 0) return 2;
    for (uint64_t f = 3; f * f <= n; f += 2)
        if (n % f == 0) return f;
    return n;
}

/* in: stride `is`; out: contiguous; tw[j] = exp(sign*2*pi*i*j/N), twstep = N/n */
static void fft_rec(const cplx *in, uint64_t is, cplx *out, uint64_t n, const cplx *tw,
                    uint64_t N, uint64_t twstep, cplx *tmp) {
    if (n == 1) { out[0] = in[0]; return; }
    uint64_t p = smallest_factor(n), m = n / p;
    if (m == 1) {
        /* direct DFT of prime length p */
        for (uint64_t k = 0; k < p; ++k) {
            double sr = 0.0, si = 0.0;
            for (uint64_t j = 0; j < p; ++j) {
                cplx w = tw[((j * k) % p) * twstep];
                cplx x = in[j * is];
                sr += x.re * w.re - x.im * w.im;
                si += x.re * w.im + x.im * w.re;
            }
            tmp[k].re = sr; tmp[k].im = si;
        }
        for (uint64_t k = 0; k < p; ++k) out[k] = tmp[k];
        return;
    }
    for (uint64_t r = 0; r < p; ++r) fft_rec(in + r * is, is * p, out + r * m, m, tw, N, twstep * p, tmp);
    cplx *t = tmp, *o = tmp + p;
    for (uint64_t k = 0; k < m; ++k) {
        for (uint64_t r = 0; r < p; ++r) {
            cplx y = out[r * m + k];
            cplx w = tw[((r * k) % n) * twstep];
            t[r].re = y.re * w.re - y.im * w.im;
            t[r].im = y.re * w.im + y.im * w.re;
        }
        for (uint64_t q = 0; q < p; ++q) {
            double sr = 0.0, si = 0.0;
            for (uint64_t r = 0; r < p; ++r) {
                cplx w = tw[((r * q * m) % n) * twstep];
                sr += t[r].re * w.re - t[r].im * w.im;
                si += t[r].re * w.im + t[r].im * w.re;
            }
            o[q].re = sr; o[q].im = si;
        }
        for (uint64_t q = 0; q < p; ++q) out[k + q * m] = o[q];
    }
}

static void fft_lines(cplx *a, uint64_t n, uint64_t count, uint64_t stride, uint64_t (*base)(uint64_t, void *),
                      void *ctx, int sign) {
    if (n == 1) return;
    cplx *tw = (cplx *)malloc(sizeof(cplx) * n);
    for (uint64_t j = 0; j < n; ++j) {
        double ang = TWOPI * (double)j / (double)n;
        tw[j].re = cos(ang);
        tw[j].im = (double)sign * sin(ang);
    }
    cplx *line = (cplx *)malloc(sizeof(cplx) * n * 2);
    cplx *res = line + n;
    cplx *tmp = (cplx *)malloc(sizeof(cplx) * (2 * n + 4));
    for (uint64_t l = 0; l < count; ++l) {
        uint64_t b = base(l, ctx);
        for (uint64_t j = 0; j < n; ++j) line[j] = a[b + j * stride];
        fft_rec(line, 1, res, n, tw, n, 1, tmp);
        for (uint64_t j = 0; j < n; ++j) a[b + j * stride] = res[j];
    }
    free(tmp); free(line); free(tw);
}

typedef struct { uint64_t nx, ny, nz; } dims3;
static uint64_t base_z(uint64_t l, void *c) { dims3 *d = (dims3 *)c; (void)d; return l * d->nz; }
static uint64_t base_y(uint64_t l, void *c) {
    dims3 *d = (dims3 *)c; uint64_t i = l / d->nz, k = l % d->nz; return i * d->ny * d->nz + k;
}
static uint64_t base_x(uint64_t l, void *c) { (void)c; return l; }

void orc_fft3d(double *data, uint64_t nx, uint64_t ny, uint64_t nz, int sign) {
    cplx *a = (cplx *)data;
    dims3 d = {nx, ny, nz};
    fft_lines(a, nz, nx * ny, 1, base_z, &d, sign);
    fft_lines(a, ny, nx * nz, nz, base_y, &d, sign);
    fft_lines(a, nx, ny * nz, ny * nz, base_x, &d, sign);
}

static void fft_components(double *data, uint64_t ncomp, const orc_settings *s, int sign, int nthreads) {
    uint64_t nc = s->gx * s->gy * s->gz;
    (void)nthreads;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads > 0 ? nthreads : 1)
    for (int64_t c = 0; c < (int64_t)ncomp; ++c) orc_fft3d(data + 2 * (uint64_t)c * nc, s->gx, s->gy, s->gz, sign);
}

/* ===================================================================== */
/* spectral solvers                                                      */
/* ===================================================================== */

/* per-cell k vector, k-hat and 1/|k|^2 exactly as the precomputed meshes */
typedef struct { double k[3], kn[3], ik2; } kpoint;
static void kpoint_at(const double *kx, const double *ky, const double *kz, uint64_t i, uint64_t j,
                      uint64_t l, uint64_t c, kpoint *kp) {
    kp->k[0] = kx[i]; kp->k[1] = ky[j]; kp->k[2] = kz[l];
    double s = k_norm_sq(kx[i], ky[j], kz[l]);
    double inv = (c == 0) ? 0.0 : inv_norm(s);
    kp->kn[0] = kx[i] * inv; kp->kn[1] = ky[j] * inv; kp->kn[2] = kz[l] * inv;
    kp->ik2 = (c == 0) ? 0.0 : inv_norm_sq(s);
}

/* update_gradient, src/flowfield/spectral_solver.rs:192-229 and
 * src/magnetic_interaction/magnetic_solver.rs:98-135: g[a][b] = (k_a * v_b) * i */
static void vector_gradient_k(const orc_settings *s, const double *v, double *g) {
    double *kx, *ky, *kz;
    uint64_t nc = s->gx * s->gy * s->gz;
    k_axes(s, &kx, &ky, &kz);
#pragma omp parallel for
    for (int64_t ii = 0; ii < (int64_t)s->gx; ++ii) {
        uint64_t i = (uint64_t)ii;
        for (uint64_t j = 0; j < s->gy; ++j)
            for (uint64_t l = 0; l < s->gz; ++l) {
                uint64_t c = (i * s->gy + j) * s->gz + l;
                double k[3] = {kx[i], ky[j], kz[l]};
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b) {
                        double vr = v[2 * (b * nc + c)], vi = v[2 * (b * nc + c) + 1];
                        /* (k + 0i) * (vr + vi i) */
                        double er = k[a] * vr - 0.0 * vi, ei = k[a] * vi + 0.0 * vr;
                        /* times i */
                        g[2 * ((uint64_t)(a * 3 + b) * nc + c)] = er * 0.0 - ei * 1.0;
                        g[2 * ((uint64_t)(a * 3 + b) * nc + c) + 1] = er * 1.0 + ei * 0.0;
                    }
            }
    }
    free(kx); free(ky); free(kz);
}

void orc_vector_gradient(const orc_settings *s, const double *bk, double *grad) {
    vector_gradient_k(s, bk, grad);
    fft_components(grad, 9, s, +1, 1);
}

/* SpectralSolver::mean_flow_field, src/flowfield/spectral_solver.rs:233-254
 * = fft_mean_flow_field (:133-189) + update_gradient (:192-229) + inverse of u */
void orc_flow_field(const orc_settings *s, const double *dist, double screening, double *u,
                    double *grad, int nthreads) {
    uint64_t nc = s->gx * s->gy * s->gz, na = s->gphi * s->gtheta;
    double *kernel = (double *)malloc(sizeof(double) * 9 * na);
    double *stress = (double *)malloc(sizeof(double) * 2 * 9 * nc);
    double *kx, *ky, *kz;
    orc_stress_kernel(s, kernel);
    orc_average_stress(s, kernel, dist, stress);
    fft_components(stress, 9, s, -1, nthreads);
    k_axes(s, &kx, &ky, &kz);
    double norm = (double)nc;
#pragma omp parallel for num_threads(nthreads > 0 ? nthreads : 1)
    for (int64_t ii = 0; ii < (int64_t)s->gx; ++ii) {
        uint64_t i = (uint64_t)ii;
        for (uint64_t j = 0; j < s->gy; ++j)
            for (uint64_t l = 0; l < s->gz; ++l) {
                uint64_t c = (i * s->gy + j) * s->gz + l;
                kpoint kp;
                kpoint_at(kx, ky, kz, i, j, l, c, &kp);
                /* sigmak = s.dot(&k): per row, sum from zero of S[r][q] * k[q] */
                double sr[3], si[3];
                for (int r = 0; r < 3; ++r) {
                    double ar = 0.0, ai = 0.0;
                    for (int q = 0; q < 3; ++q) {
                        double xr = stress[2 * ((uint64_t)(r * 3 + q) * nc + c)];
                        double xi = stress[2 * ((uint64_t)(r * 3 + q) * nc + c) + 1];
                        ar = ar + (xr * kp.k[q] - xi * 0.0);
                        ai = ai + (xr * 0.0 + xi * kp.k[q]);
                    }
                    sr[r] = ar; si[r] = ai;
                }
                /* ksigmak = kn.dot(&sigmak) */
                double kr = 0.0, ki = 0.0;
                for (int r = 0; r < 3; ++r) {
                    kr = kr + (kp.kn[r] * sr[r] - 0.0 * si[r]);
                    ki = ki + (kp.kn[r] * si[r] + 0.0 * sr[r]);
                }
                /* sigmak -= kn * ksigmak ; *= (ik2 + screening)/norm ; *= i */
                double fac = (kp.ik2 + screening) / norm;
                for (int r = 0; r < 3; ++r) {
                    double tr = sr[r] - (kp.kn[r] * kr - 0.0 * ki);
                    double ti = si[r] - (kp.kn[r] * ki + 0.0 * kr);
                    double mr = tr * fac - ti * 0.0, mi = ti * fac + tr * 0.0;
                    u[2 * (r * nc + c)] = mr * 0.0 - mi * 1.0;
                    u[2 * (r * nc + c) + 1] = mi * 0.0 + mr * 1.0;
                }
            }
    }
    vector_gradient_k(s, u, grad);
    fft_components(grad, 9, s, +1, nthreads);
    fft_components(u, 3, s, +1, nthreads);
    free(kx); free(ky); free(kz);
    free(stress); free(kernel);
}

/* MagneticSolver::mean_magnetic_field, src/magnetic_interaction/magnetic_solver.rs:139-161
 * = fft_mean_magnetic_field (:71-95, k = 0 mode kept) + update_gradient + inverse of B */
void orc_magnetic_field(const orc_settings *s, const double *dist, double *b, double *gradb,
                        int nthreads) {
    uint64_t nc = s->gx * s->gy * s->gz;
    double *kx, *ky, *kz;
    orc_director_field(s, dist, b);
    fft_components(b, 3, s, -1, nthreads);
    k_axes(s, &kx, &ky, &kz);
    double norm = (double)nc;
#pragma omp parallel for num_threads(nthreads > 0 ? nthreads : 1)
    for (int64_t ii = 0; ii < (int64_t)s->gx; ++ii) {
        uint64_t i = (uint64_t)ii;
        for (uint64_t j = 0; j < s->gy; ++j)
            for (uint64_t l = 0; l < s->gz; ++l) {
                uint64_t c = (i * s->gy + j) * s->gz + l;
                kpoint kp;
                kpoint_at(kx, ky, kz, i, j, l, c, &kp);
                double dr = 0.0, di = 0.0;
                for (int r = 0; r < 3; ++r) {
                    double pr = b[2 * (r * nc + c)], pi = b[2 * (r * nc + c) + 1];
                    dr = dr + (kp.kn[r] * pr - 0.0 * pi);
                    di = di + (kp.kn[r] * pi + 0.0 * pr);
                }
                for (int r = 0; r < 3; ++r) {
                    double pr = b[2 * (r * nc + c)], pi = b[2 * (r * nc + c) + 1];
                    double tr = pr - (kp.kn[r] * dr - 0.0 * di);
                    double ti = pi - (kp.kn[r] * di + 0.0 * dr);
                    b[2 * (r * nc + c)] = tr / norm;
                    b[2 * (r * nc + c) + 1] = ti / norm;
                }
            }
    }
    vector_gradient_k(s, b, gradb);
    fft_components(gradb, 9, s, +1, nthreads);
    fft_components(b, 3, s, +1, nthreads);
    free(kx); free(ky); free(kz);
}

/* ===================================================================== */
/* trilinear interpolation, src/mesh/interpolate.rs                      */
/* ===================================================================== */

/* lerp 0.2.0: a * (1 - t) + b * t */
static double lerp(double a, double b, double t) { return a * (1.0 - t) + b * t; }

static uint64_t wrap_idx(int64_t i, uint64_t n) { return (uint64_t)((i + (int64_t)n) % (int64_t)n); }

void orc_interpolate(const orc_settings *s, const double *field, int ncomp, const double p[3], int zbug,
                     double *out) {
    double gw[5];
    orc_grid_width(s, gw);
    uint64_t nc = s->gx * s->gy * s->gz;
    /* relative position, interpolate.rs:19-23 (Rust % on f64 is fmod) */
    double fx = fmod(p[0] / gw[0] + 0.5, 1.0);
    double fy = fmod(p[1] / gw[1] + 0.5, 1.0);
    double fz = fmod((zbug ? p[1] : p[2]) / gw[2] + 0.5, 1.0);
    /* lower corner, get_neighbouring_cell_values :68-78: floor(p / gw - 0.5) */
    int64_t ix = (int64_t)floor(p[0] / gw[0] - 0.5);
    int64_t iy = (int64_t)floor(p[1] / gw[1] - 0.5);
    int64_t iz = (int64_t)floor(p[2] / gw[2] - 0.5);
    for (int c = 0; c < ncomp; ++c) {
        const double *f = field + (uint64_t)c * nc;
        double v[2][2][2];
        for (int a = 0; a < 2; ++a)
            for (int b = 0; b < 2; ++b)
                for (int d = 0; d < 2; ++d) {
                    uint64_t i = wrap_idx(ix + a, s->gx), j = wrap_idx(iy + b, s->gy), k = wrap_idx(iz + d, s->gz);
                    v[a][b][d] = f[(i * s->gy + j) * s->gz + k];
                }
        /* trilinear_interpolation :104-119 */
        double c00 = lerp(v[0][0][0], v[1][0][0], fx);
        double c01 = lerp(v[0][0][1], v[1][0][1], fx);
        double c10 = lerp(v[0][1][0], v[1][1][0], fx);
        double c11 = lerp(v[0][1][1], v[1][1][1], fx);
        double c0 = lerp(c00, c10, fy);
        double c1 = lerp(c01, c11, fy);
        out[c] = lerp(c0, c1, fz);
    }
}

/* ===================================================================== */
/* Langevin builder, src/integrators/langevin_builder/{mod.rs,modifiers.rs} */
/* ===================================================================== */

/* ndarray Array2.dot(Array1) row: unrolled_dot of length 3 = ((0+a0b0)+a1b1)+a2b2 */
static double row_dot3(const double *m, const double *v) {
    double s = 0.0;
    s = s + m[0] * v[0];
    s = s + m[1] * v[1];
    s = s + m[2] * v[2];
    return s;
}
/* NumVector::dot, src/vector/mod.rs:51-53: map(a*b).sum() folding from 0.0 */
static double vec_dot(const double *a, const double *b) {
    double s = 0.0;
    s = s + a[0] * b[0];
    s = s + a[1] * b[1];
    s = s + a[2] * b[2];
    return s;
}
/* vecmath 0.3.1 vec3_dot / vec3_cross */
static double vm_dot(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static void vm_cross(const double *a, const double *b, double *o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}
/* quaternion 0.3.1 mul: (a0*b0 - dot(a1,b1), (b1*a0 + a1*b0) + cross(a1,b1)) */
static void q_mul(double a0, const double *a1, double b0, const double *b1, double *o0, double *o1) {
    double c[3];
    vm_cross(a1, b1, c);
    *o0 = a0 * b0 - vm_dot(a1, b1);
    for (int i = 0; i < 3; ++i) o1[i] = (b1[i] * a0 + a1[i] * b0) + c[i];
}

void orc_langevin(const double p[5], uint32_t mask, const orc_langevin_args *a, double out[5]) {
    /* LangevinBuilder::new, mod.rs:25-38 with CosSinOrientation, particle.rs:155-173 */
    double cp = cos(p[3]), sp = sin(p[3]), ct = cos(p[4]), st = sin(p[4]);
    double pos[3] = {p[0], p[1], p[2]};
    double n[3] = {st * cp, st * sp, ct};
    double dp[3] = {0., 0., 0.}, dn[3] = {0., 0., 0.};
    int k;

    if (mask & ORC_SELF_PROPULSION)  /* modifiers.rs:39-46 */
        for (k = 0; k < 3; ++k) { dp[k] = dp[k] + n[k]; dn[k] = dn[k] + 0.0; }
    if (mask & ORC_CONVECTION)  /* modifiers.rs:49-56 */
        for (k = 0; k < 3; ++k) { dp[k] = dp[k] + a->flow[k]; dn[k] = dn[k] + 0.0; }
    if (mask & ORC_MDD_FORCE) {  /* modifiers.rs:59-70, magnetic_interaction/mod.rs:13-17 */
        double f[3];
        for (k = 0; k < 3; ++k) f[k] = row_dot3(a->gradb + 3 * k, n);
        for (k = 0; k < 3; ++k) { dp[k] = dp[k] + f[k] * a->drag; dn[k] = dn[k] + 0.0; }
    }
    if (mask & ORC_EXTERNAL_FIELD) {  /* modifiers.rs:103-119, field along y */
        double b[3] = {0., a->reorientation, 0.};
        double d = vec_dot(n, b);
        for (k = 0; k < 3; ++k) b[k] -= n[k] * d;
        for (k = 0; k < 3; ++k) { dp[k] = dp[k] + 0.0; dn[k] = dn[k] + b[k]; }
    }
    if (mask & ORC_MDD_ROTATION) {  /* modifiers.rs:172-187 */
        double b[3] = {a->b[0], a->b[1], a->b[2]};
        double d = vec_dot(n, b);
        for (k = 0; k < 3; ++k) b[k] -= n[k] * d;
        for (k = 0; k < 3; ++k) { dp[k] = dp[k] + 0.0; dn[k] = dn[k] + b[k]; }
    }
    if (mask & ORC_JEFFREY_VORTICITY) {  /* modifiers.rs:123-143 */
        double f[3];
        for (k = 0; k < 3; ++k) f[k] = row_dot3(a->vort + 3 * k, n) * (-1.);
        for (k = 0; k < 3; ++k) { dp[k] = dp[k] + 0.0; dn[k] = dn[k] + f[k]; }
    }
    if (mask & ORC_JEFFREY_STRAIN) {  /* modifiers.rs:147-170 */
        double f[3];
        for (k = 0; k < 3; ++k) f[k] = row_dot3(a->strain + 3 * k, n);
        for (k = 0; k < 3; ++k) f[k] *= a->shape;
        double fn = row_dot3(f, n);
        for (k = 0; k < 3; ++k) f[k] -= n[k] * fn;
        for (k = 0; k < 3; ++k) { dp[k] = dp[k] + 0.0; dn[k] = dn[k] + f[k]; }
    }
    if (mask & ORC_STEP)  /* mod.rs:114-119 */
        for (k = 0; k < 3; ++k) { dp[k] = dp[k] * a->dt; dn[k] = dn[k] * a->dt; }
    if (mask & ORC_TRANS_DIFFUSION)  /* modifiers.rs:86-99 */
        for (k = 0; k < 3; ++k) { dp[k] = dp[k] + a->xi[k] * a->diff; dn[k] = dn[k] + 0.0; }
    if (mask & ORC_ROT_DIFFUSION) {  /* modifiers.rs:199-231 */
        double ca = cos(a->axis_angle), sa = sin(a->axis_angle);
        double ax[3] = {cp * ct * sa - ca * sp, ca * cp + ct * sa * sp, -sa * st};
        /* quaternion::axis_angle: half = angle / 2 */
        double half = a->rotate_angle / (1.0 + 1.0);
        double q0 = cos(half), sh = sin(half);
        double q1[3] = {ax[0] * sh, ax[1] * sh, ax[2] * sh};
        /* rotate_vector: mul(mul(q, (0, v)), conj(q)).1 */
        double t0, t1[3], r0, r1[3], qc[3] = {-q1[0], -q1[1], -q1[2]};
        q_mul(q0, q1, 0.0, n, &t0, t1);
        q_mul(t0, t1, q0, qc, &r0, r1);
        for (k = 0; k < 3; ++k) { dp[k] = dp[k] + 0.0; dn[k] = dn[k] + (r1[k] - n[k]); }
    }
    /* finalize, mod.rs:121-125: Particle::from(old + delta), then pbc */
    double np[3], nv[3], o[2];
    for (k = 0; k < 3; ++k) { np[k] = pos[k] + dp[k]; nv[k] = n[k] + dn[k]; }
    orc_from_vector(nv, o);
    out[0] = orc_modulo(np[0], a->bx);
    out[1] = orc_modulo(np[1], a->by);
    out[2] = orc_modulo(np[2], a->bz);
    double ap[2];
    orc_ang_pbc(o[0], o[1], ap);
    out[3] = ap[0];
    out[4] = ap[1];
}

/* ===================================================================== */
/* whole simulation: Simulation::{new, init, do_timestep},               */
/* src/bin/simulation/mod.rs:91-374                                      */
/* ===================================================================== */

struct orc_sim {
    orc_settings s;
    uint64_t n, ncell, nbins, timestep;
    int nthreads;
    double *particles, *dist, *noise;
    double *u, *grad, *b, *gradb, *dens;
    double *vort, *strain;  /* real parts of W and E, [3][3][ncell] */
    double *re_u, *re_b, *re_gradb;  /* real parts for the trilinear gather */
    uint64_t *rng;          /* PCG32 state per thread (baseline noise only) */
};

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

orc_sim *orc_sim_new(const orc_settings *s, uint64_t n, int nthreads) {
    orc_sim *sim = (orc_sim *)calloc(1, sizeof(orc_sim));
    sim->s = *s;
    sim->n = n;
    sim->ncell = s->gx * s->gy * s->gz;
    sim->nbins = sim->ncell * s->gphi * s->gtheta;
    sim->nthreads = nthreads > 0 ? nthreads : 1;
    sim->particles = (double *)calloc(5 * (n ? n : 1), sizeof(double));
    sim->noise = (double *)calloc(5 * (n ? n : 1), sizeof(double));
    sim->dist = (double *)calloc(sim->nbins, sizeof(double));
    sim->u = (double *)calloc(2 * 3 * sim->ncell, sizeof(double));
    sim->grad = (double *)calloc(2 * 9 * sim->ncell, sizeof(double));
    sim->b = (double *)calloc(2 * 3 * sim->ncell, sizeof(double));
    sim->gradb = (double *)calloc(2 * 9 * sim->ncell, sizeof(double));
    sim->dens = (double *)calloc(sim->ncell, sizeof(double));
    sim->vort = (double *)calloc(9 * sim->ncell, sizeof(double));
    sim->strain = (double *)calloc(9 * sim->ncell, sizeof(double));
    sim->re_u = (double *)calloc(3 * sim->ncell, sizeof(double));
    sim->re_b = (double *)calloc(3 * sim->ncell, sizeof(double));
    sim->re_gradb = (double *)calloc(9 * sim->ncell, sizeof(double));
    /* every thread's generator seeded with the same seed, like
     * src/bin/simulation/mod.rs:126-128 */
    sim->rng = (uint64_t *)calloc(2 * (uint64_t)sim->nthreads, sizeof(uint64_t));
    for (int t = 0; t < sim->nthreads; ++t) {
        sim->rng[2 * t] = s->seed * 6364136223846793005ULL + 1442695040888963407ULL;
        sim->rng[2 * t + 1] = 1442695040888963407ULL | 1ULL;
    }
    return sim;
}

void orc_sim_free(orc_sim *sim) {
    if (!sim) return;
    free(sim->particles); free(sim->noise); free(sim->dist); free(sim->u); free(sim->grad);
    free(sim->b); free(sim->gradb); free(sim->dens); free(sim->vort); free(sim->strain);
    free(sim->re_u); free(sim->re_b); free(sim->re_gradb);
    free(sim->rng);
    free(sim);
}

static void sample_scaled(orc_sim *sim) {
    /* distribution.sample_from + *= Lx*Ly*Lz, src/bin/simulation/mod.rs:253-257 */
    orc_sample_from(&sim->s, sim->particles, sim->n, sim->dist);
    double v = sim->s.bx * sim->s.by * sim->s.bz;
    for (uint64_t i = 0; i < sim->nbins; ++i) sim->dist[i] *= v;
}

/* Simulation::init, src/bin/simulation/mod.rs:163-196 */
int orc_sim_init(orc_sim *sim, const double *particles, uint64_t n) {
    if (n != sim->n) return -1;
    for (uint64_t i = 0; i < n; ++i) orc_particle_new(&sim->s, particles + 5 * i, sim->particles + 5 * i);
    sample_scaled(sim);
    return 0;
}

/* PCG32 (O'Neill 2014, XSH-RR) for the timed baseline's own noise */
static uint32_t pcg32(uint64_t *st) {
    uint64_t old = st[0];
    st[0] = old * 6364136223846793005ULL + st[1];
    uint32_t x = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t r = (uint32_t)(old >> 59u);
    return (x >> r) | (x << ((32u - r) & 31u));
}
static double pcg_uniform(uint64_t *st) {
    uint64_t a = pcg32(st), b = pcg32(st);
    return (double)(((a << 32) | b) >> 11) * (1.0 / 9007199254740992.0);
}
static double pcg_normal(uint64_t *st) {
    /* Marsaglia polar method */
    for (;;) {
        double u = 2.0 * pcg_uniform(st) - 1.0, v = 2.0 * pcg_uniform(st) - 1.0;
        double q = u * u + v * v;
        if (q > 0.0 && q < 1.0) return u * sqrt(-2.0 * log(q) / q);
    }
}

static void generate_noise(orc_sim *sim) {
    /* src/bin/simulation/mod.rs:259-286: chunks of n/threads+1 per thread */
    double dr = sqrt(2. * sim->s.rot_diff * sim->s.timestep);
    uint64_t chunk = sim->n / (uint64_t)sim->nthreads + 1;
#pragma omp parallel for num_threads(sim->nthreads) schedule(static, 1)
    for (int t = 0; t < sim->nthreads; ++t) {
        /* thread-local copy of the generator state: no false sharing */
        uint64_t st[2] = {sim->rng[2 * t], sim->rng[2 * t + 1]};
        uint64_t lo = (uint64_t)t * chunk, hi = lo + chunk;
        if (hi > sim->n) hi = sim->n;
        for (uint64_t i = lo; i < hi; ++i) {
            double *r = sim->noise + 5 * i;
            r[0] = pcg_normal(st);
            r[1] = pcg_normal(st);
            r[2] = pcg_normal(st);
            r[3] = TWOPI * pcg_uniform(st);
            r[4] = dr * sqrt(-2. * log(1. - pcg_uniform(st)));
        }
        sim->rng[2 * t] = st[0];
    }
}

/* Simulation::do_timestep, src/bin/simulation/mod.rs:251-374 */
uint64_t orc_sim_step(orc_sim *sim, const double *noise) {
    const orc_settings *s = &sim->s;
    uint64_t nc = sim->ncell, na = s->gphi * s->gtheta;
    double gw[5];
    orc_grid_width(s, gw);

    sample_scaled(sim);
    if (noise) memcpy(sim->noise, noise, sizeof(double) * 5 * sim->n);
    else generate_noise(sim);

    orc_magnetic_field(s, sim->dist, sim->b, sim->gradb, sim->nthreads);
    orc_flow_field(s, sim->dist, s->hydro_screening, sim->u, sim->grad, sim->nthreads);

    /* W = (G - G^T)*0.5, E = (G + G^T)*0.5 (real parts), mod.rs:302-308 */
    for (uint64_t c = 0; c < nc; ++c)
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                double gab = sim->grad[2 * ((uint64_t)(a * 3 + b) * nc + c)];
                double gba = sim->grad[2 * ((uint64_t)(b * 3 + a) * nc + c)];
                sim->vort[(uint64_t)(a * 3 + b) * nc + c] = (gab - gba) * 0.5;
                sim->strain[(uint64_t)(a * 3 + b) * nc + c] = (gab + gba) * 0.5;
            }
    for (uint64_t c = 0; c < nc; ++c) {
        for (int k = 0; k < 3; ++k) {
            sim->re_u[k * nc + c] = sim->u[2 * (k * nc + c)];
            sim->re_b[k * nc + c] = sim->b[2 * (k * nc + c)];
        }
        for (int k = 0; k < 9; ++k) sim->re_gradb[k * nc + c] = sim->gradb[2 * (k * nc + c)];
    }
    /* dens = sum over angles (sequential) * dtheta*dphi, mod.rs:312-316 */
    double dthph = gw[4] * gw[3];
    for (uint64_t c = 0; c < nc; ++c) {
        double acc = 0.0;
        for (uint64_t a = 0; a < na; ++a) acc = acc + sim->dist[c * na + a];
        sim->dens[c] = acc * dthph;
    }

    /* particle loop, mod.rs:318-369 */
#pragma omp parallel for num_threads(sim->nthreads) schedule(static)
    for (int64_t ii = 0; ii < (int64_t)sim->n; ++ii) {
        uint64_t i = (uint64_t)ii;
        double *p = sim->particles + 5 * i;
        const double *r = sim->noise + 5 * i;
        uint64_t g[3];
        orc_cell_index(s, p, g);
        uint64_t c = (g[0] * s->gy + g[1]) * s->gz + g[2];
        orc_langevin_args a;
        double dens;
        if (s->gather == 0) {
            for (int k = 0; k < 3; ++k) {
                a.flow[k] = sim->u[2 * (k * nc + c)];
                a.b[k] = sim->b[2 * (k * nc + c)] * s->magnetic_dipole_dipole;
            }
            for (int k = 0; k < 9; ++k) {
                a.vort[k] = sim->vort[(uint64_t)k * nc + c];
                a.strain[k] = sim->strain[(uint64_t)k * nc + c];
                a.gradb[k] = sim->gradb[2 * ((uint64_t)k * nc + c)];
            }
            dens = sim->dens[c];
        } else {
            /* every gathered field interpolated at the particle position */
            int zb = s->gather == 2;
            double bi[3];
            orc_interpolate(s, sim->re_u, 3, p, zb, a.flow);
            orc_interpolate(s, sim->vort, 9, p, zb, a.vort);
            orc_interpolate(s, sim->strain, 9, p, zb, a.strain);
            orc_interpolate(s, sim->re_b, 3, p, zb, bi);
            orc_interpolate(s, sim->re_gradb, 9, p, zb, a.gradb);
            orc_interpolate(s, sim->dens, 1, p, zb, &dens);
            for (int k = 0; k < 3; ++k) a.b[k] = bi[k] * s->magnetic_dipole_dipole;
        }
        for (int k = 0; k < 3; ++k) a.xi[k] = r[k];
        double volex = s->volume_exclusion * dens;
        a.drag = s->magnetic_drag;
        a.reorientation = s->magnetic_reorientation;
        a.shape = s->shape;
        a.dt = s->timestep;
        a.diff = sqrt(2. * s->timestep * (s->trans_diff + volex));
        a.axis_angle = r[3];
        a.rotate_angle = r[4];
        a.bx = s->bx; a.by = s->by; a.bz = s->bz;
        double out[5];
        orc_langevin(p, ORC_ALL, &a, out);
        if (s->quasi2d) {
            out[2] = 0.0;
            out[4] = PI / 2.;
        }
        for (int k = 0; k < 5; ++k) p[k] = out[k];
    }
    sim->timestep += 1;
    return sim->timestep;
}

double *orc_sim_particles(orc_sim *sim) { return sim->particles; }
double *orc_sim_distribution(orc_sim *sim) { return sim->dist; }
double *orc_sim_flow(orc_sim *sim) { return sim->u; }
double *orc_sim_flow_grad(orc_sim *sim) { return sim->grad; }
double *orc_sim_mag(orc_sim *sim) { return sim->b; }
double *orc_sim_mag_grad(orc_sim *sim) { return sim->gradb; }
double *orc_sim_density(orc_sim *sim) { return sim->dens; }
double *orc_sim_noise(orc_sim *sim) { return sim->noise; }
uint64_t orc_sim_timestep(const orc_sim *sim) { return sim->timestep; }
void orc_sim_set_timestep(orc_sim *sim, uint64_t t) { sim->timestep = t; }
