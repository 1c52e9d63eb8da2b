// mixed.cuh -- parameters and launch wrappers of the FP32 mixed-precision
// timestep (mixed.cu).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <vector>

#include "../../include/ssgpu.h"
#include "common.cuh"

namespace ss {

struct MixedParams {
    int gx, gy, gz, gphi, gtheta;
    int ncell, nang;
    unsigned long long n;
    double bx, by, bz;  // positions stay FP64 (or 64-bit fixed point)
    double bx2, by2, bz2;  // 2 L, for the exact wrap
    float igwf[5];      // 1 / grid width, FP32 binning
    float gwf[3];       // grid width (FP32), to skip the wrap test in interior cells
    float s32[3];       // 2^32 / L: FP32 step -> fixed-point increment
    double unit[3];     // L / 2^64: fixed point -> FP64
    double dist_den, volume;
    float measure, dthph, two_dt, Dt, volex, dt;
    float drag, reorient, shape, mdd, sigma_rot;
    unsigned long long seed;
    uint32_t mask;
    int hdim[3];  // half-spectrum shape of the real-to-complex transforms (as DevParams)
    int nhalf;
    int cstride;  // component stride of the contraction's real fields (as DevParams)
};

// id == nullptr: leave id as it is (rows already sorted, id holds their caller indices)
void launch_ingest_m(cudaStream_t s, bool fixed, const double *aos, unsigned long long n, const DevParams &P,
                     const MixedParams &M, double *const xs[3], float *const as[2], uint32_t *id);
void launch_egest_m(cudaStream_t s, bool fixed, unsigned long long n, const MixedParams &M, double *const xs[3],
                    float *const as[2], const uint32_t *id, double *aos);
void launch_bin_m(cudaStream_t s, bool fixed, unsigned long long n, const MixedParams &M, double *const xs[3],
                  float *const as[2], uint32_t *key, uint32_t *counts);
// the FP32 angular contraction (contract.cu): real fwd [12][cstride], the
// table's diffusion length and the FP64 component sums (sums[0..9) with
// stress, sums[9..12) with the polarisation) in a fixed order.  partials:
// contract_m_blocks(ncell, sms) x 12 float pairs; done: a counter that is 0
// between launches; sms: multiprocessors of the device.  dist != nullptr: an
// FP32 distribution times fscale replaces the counts (the denoised histogram).
// With a tensor map of the source (make_bins_tmap), the transposed angle
// kernels (kernel_transposed) and an error word, the TMA-staged kernel runs;
// err gets bit 0x100 when one of its copies timed out.
unsigned contract_m_blocks(int ncell, int sms);
void launch_contract_m(cudaStream_t s, bool stress, bool mag, const uint32_t *counts, const float *kern,
                       const MixedParams &M, float *fwd, float *table, int tstride, float2 *partials,
                       unsigned *done, double *sums, int sms, const float *dist = nullptr, float fscale = 0.f,
                       const CUtensorMap *tmap = nullptr, const float *kern_t = nullptr, unsigned *err = nullptr);
void kernel_transposed(const std::vector<double> &K, int na, std::vector<float> &out);
bool make_bins_tmap(CUtensorMap *map, const void *base, int ncell, int na);
bool contract_tma_fits(int na);
void launch_counts_to_unit(cudaStream_t s, const uint32_t *counts, long long nbins, float inv_mean, float *x);
// the FP64 means removed from the real fields fr [comp][cstride], components c0 .. c1
void launch_center_m(cudaStream_t s, float *fr, int c0, int c1, int ncell, int cstride, const double *sums);
// the k-space operators on the half spectrum, Hermitian part (or with anti the
// anti-Hermitian part); as launch_kspace of the FP64 path
void launch_kspace_m(cudaStream_t s, bool flow, bool mag, bool anti, const float2 *fwd, float2 *inv,
                     const MixedParams &M, float screening);
void launch_table_m(cudaStream_t s, bool flow, bool mag, const float *inv, const MixedParams &M, float *table,
                    int tstride, const double *sums);
// complex FP64 fields dst [comp][cell] from FP32 real parts re and imaginary
// parts im (null: zero), the FP64 mean added to components m0 .. m1
void launch_widen_m(cudaStream_t s, const float *re, const float *im, long long count, int ncell, int comp0, int m0,
                    int m1, const double *sums, double2 *dst);
void launch_real_to_complex_f(cudaStream_t s, const float *src, int count, int sstride, float2 *dst);
void launch_complex_to_real_f(cudaStream_t s, const float2 *src, int count, float *dst);
// counting sort of the resident particles by their cell keys into the other buffer set (4 launches)
void launch_resort_m(cudaStream_t s, const MixedParams &M, double *const xs[3], float *const as[2], const uint32_t *key,
                     const uint32_t *id, double *const xd[3], float *const ad[2], uint32_t *keyd, uint32_t *idd,
                     uint32_t *cellcount, uint32_t *cursor);
void launch_update_m(cudaStream_t s, bool fixed, bool q2d, bool canon, bool mag, bool host_noise, const MixedParams &M,
                     double *const xs[3], float *const as[2], uint32_t *key, const uint32_t *id, const float *table,
                     const double *noise, const unsigned long long *d_step, uint32_t *counts_next);
void launch_noise_m(cudaStream_t s, bool q2d, const MixedParams &M, unsigned long long t, double *out);

// host side, defined in ssgpu.cu and shared with the ensemble: the FP64 angle
// kernels [component][phi][theta], 9 stress components then the 3
// orientation components, and the context-free error of ss_last_error
void build_angle_kernels(const ss_grid &grid, const ss_params &prm, std::vector<double> &K);
void record_error(const char *msg);

}  // namespace ss
