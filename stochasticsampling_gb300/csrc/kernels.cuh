// kernels.cuh -- launch wrappers of the timestep kernels (kernels.cu).
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "common.cuh"

namespace ss {

void launch_scan_rows(cudaStream_t s, const double *aos, unsigned long long n, unsigned long long *scan);
void launch_egest(cudaStream_t s, unsigned long long n, double *const xs[5], const uint32_t *id, double *aos);
// k_ingest_bin plus the row checks of k_scan_rows on rows off .. off + n
// (aos, xs, id, key point at row off)
void launch_ingest_bin_check(cudaStream_t s, const double *aos, unsigned long long n, unsigned long long off,
                             const DevParams &P, double *const xs[5], uint32_t *id, uint32_t *key,
                             uint32_t *counts, unsigned long long *scan, uint32_t *err);
// counting sort of host-layout rows by spatial cell: sorted[pos] = aos[i],
// orig[pos] = i (cellkey, cellcount, cursor: scratch of n, ncell, ncell)
void launch_sort_rows(cudaStream_t s, const double *aos, unsigned long long n, const DevParams &P,
                      uint32_t *cellkey, uint32_t *cellcount, uint32_t *cursor, double *sorted, uint32_t *orig);
// Particle::new and the first histogram in one pass (canon: every row in the canonical quasi-2-D state);
// id == nullptr leaves id as it is
void launch_ingest_bin(cudaStream_t s, bool canon, const double *aos, unsigned long long n, const DevParams &P,
                       double *const xs[5], uint32_t *id, uint32_t *key, uint32_t *counts, uint32_t *err);
void launch_counts_to_dist(cudaStream_t s, const uint32_t *counts, const DevParams &P, double *dist);
// the contraction of a distribution (or of counts): real fields fwd [12][ncell]
void launch_contract(cudaStream_t s, bool stress, bool mag, const uint32_t *counts, const double *dist,
                     const double *lut, int lut_n, const double *kern, const DevParams &P, double *fwd,
                     double *table, int tstride, uint32_t *cellcount);
// the FP64 contraction of a histogram (contract.cu): kslice, factor from
// kernel_slices; kern and lut serve cells of more than 2^12 particles
void launch_contract_x(cudaStream_t s, bool stress, bool mag, const uint32_t *counts, const float *kslice,
                       const double *factor, const double *kern, const double *lut, int lut_n, const DevParams &P,
                       double *fwd, double *table, int tstride, uint32_t *cellcount);
// host: the angle kernels K [12][na] as four 12-bit integer slices per entry,
// slices [na][48] (component j, slice s at 4 j + s), and per component the
// factor 2^(E_j - 48) * measure_v_over_d that turns the combined slice sums
// into the contraction
void kernel_slices(const std::vector<double> &K, int na, double measure_v_over_d, std::vector<float> &slices,
                   std::vector<double> &factor);
// shared-memory limits of the contraction kernels on the current device
cudaError_t contract_prepare();
// the k-space operators on the half spectrum (fwd [12][nhalf] -> inv
// [24][nhalf]): their Hermitian part, or with anti the anti-Hermitian part
// (the imaginary parts of the reference's complex fields)
void launch_kspace(cudaStream_t s, bool flow, bool mag, bool anti, const double2 *fwd, double2 *inv,
                   const DevParams &P, double screening);
// one-cell grids: src values sstride apart -> complex (value, 0)
void launch_real_to_complex(cudaStream_t s, const double *src, int count, int sstride, double2 *dst);
void launch_complex_to_real(cudaStream_t s, const double2 *src, int count, double *dst);
void launch_combine_complex(cudaStream_t s, const double *re, const double *im, long long count, double2 *dst);
// the per-cell field rows from the real fields inv [24][ncell]
void launch_table(cudaStream_t s, bool flow, bool mag, const double *inv, const DevParams &P, double *table,
                  int tstride, double *ctab);
// canon: quasi2d with every particle in the canonical state (z = 0, theta = pi/2);
// ctab: the canonical table of the step (k_table), or null
void launch_update(cudaStream_t s, bool q2d, bool canon, bool mag, bool host_noise, const DevParams &P,
                   double *const xs[5], uint32_t *key, const uint32_t *id, const double *table, const double *ctab,
                   const double *noise, const unsigned long long *d_step, uint32_t *counts_next, uint32_t *err);
void launch_step_inc(cudaStream_t s, unsigned long long *d_step);
void launch_sample_initial(cudaStream_t s, bool homogeneous, const DevParams &P, double kappa, double *aos,
                           uint32_t *err);
void launch_noise(cudaStream_t s, bool q2d, const DevParams &P, unsigned long long t, double *out);
void launch_scan(cudaStream_t s, const uint32_t *cnt, int n, uint32_t *out);
void launch_scatter(cudaStream_t s, unsigned long long n, double *const src[5], const uint32_t *key,
                    const uint32_t *id, double *const dst[5], uint32_t *key2, uint32_t *id2, uint32_t *cursor);
void launch_zero_u32(cudaStream_t s, uint32_t *p, long long n);
void launch_real_parts(cudaStream_t s, const double2 *src, long long count, double *dst);
void launch_half_pi(cudaStream_t s, double *out);
void launch_langevin_args(cudaStream_t s, const double *in, unsigned long long n, uint32_t mask, const double *args,
                          double *out);
// blocks x 256 threads, 8 FMA chains of iters steps each; out[blocks * 256]
void launch_fp64_rate(cudaStream_t s, unsigned blocks, int iters, double *out);

}  // namespace ss
