// noalloc.cu -- the distribution of a particle list without any allocation.
//
// Some callers cannot call cudaMalloc or cudaFree at the point where they
// need a histogram: a hook called from another library's loop, where the
// device-wide synchronisation of cudaFree would stall or deadlock that loop,
// or an application that reserves a fixed device-memory budget at start-up
// and may not grow it afterwards.  ss_sample_distribution_noalloc serves
// them: its only scratch is the file-scope device array below, of a fixed
// size, which every GPU that loads this library holds until the process
// exits.  It allocates nothing.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <mutex>
#include <string>

#include "../../include/ssgpu.h"
#include "common.cuh"

using namespace ss;

namespace ss {
void record_error(const char *msg);  // ssgpu.cu: the context-free error of ss_last_error
}

namespace {

// scratch: one u32 count per bin, then the error word (index
// SS_NOALLOC_MAX_BINS: non-zero when a row had a non-finite coordinate),
// shared by every call on a device
constexpr unsigned kErrWord = SS_NOALLOC_MAX_BINS;
static __device__ __align__(256) uint32_t g_noalloc_counts[SS_NOALLOC_MAX_BINS + 64];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
uint32_t *g_counts_ptr[kMaxDevices] = {};
int g_sms[kMaxDevices] = {};  // multiprocessors of each device, looked up with the address

// the message is returned by ss_last_error(NULL, ...)
int noalloc_fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    ss::record_error(buf);
    return code;
}

// device address of the scratch array on the current device and the
// device's multiprocessor count, looked up once per device with that device
// current
int scratch_on_current_device(uint32_t **out, int *sms) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return noalloc_fail(SS_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return noalloc_fail(SS_ERR_CUDA, "device index %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_counts_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_counts);
        if (e != cudaSuccess)
            return noalloc_fail(SS_ERR_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
        int m = 0;
        e = cudaDeviceGetAttribute(&m, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess)
            return noalloc_fail(SS_ERR_CUDA, "cudaDeviceGetAttribute(multiprocessors): %s", cudaGetErrorString(e));
        g_sms[dev] = m > 0 ? m : 1;
        g_counts_ptr[dev] = static_cast<uint32_t *>(p);
    }
    *out = g_counts_ptr[dev];
    *sms = g_sms[dev];
    return SS_OK;
}

// the counts of the call's bins and the error word to zero
__global__ void k_noalloc_zero(uint32_t *__restrict__ counts, long long nbins) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    long long stride = (long long)gridDim.x * blockDim.x;
    if (i == 0) counts[kErrWord] = 0u;
    for (; i < nbins; i += stride) counts[i] = 0u;
}

// Particle::new (src/particle.rs:186-201) on each row, then the bin of
// Distribution::coord_to_grid, counted with an atomic add.  A row with a
// non-finite coordinate (which ss_init refuses) is not counted; it sets the
// error word instead.
__global__ void k_noalloc_bin(const double *__restrict__ aos, unsigned long long n, DevParams P,
                              uint32_t *__restrict__ counts) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double *p = aos + 5 * i;
    const unsigned long long *b = reinterpret_cast<const unsigned long long *>(p);
    bool bad = false;
#pragma unroll
    for (int k = 0; k < 5; ++k) bad |= ((b[k] >> 52) & 0x7FFull) == 0x7FFull;  // Inf or NaN
    if (bad) {
        atomicOr(counts + kErrWord, 1u);
        return;
    }
    double x = ref_modulo(p[0], P.bx), y = ref_modulo(p[1], P.by), z = ref_modulo(p[2], P.bz);
    double ph = p[3], th = p[4];
    ref_ang_pbc(ph, th);
    x = ref_modulo(x, P.bx);
    y = ref_modulo(y, P.by);
    z = ref_modulo(z, P.bz);
    ref_ang_pbc(ph, th);
    uint32_t err = 0;
    int ix = ref_bin(x, P.gw[0], P.igw[0], P.gx, err);
    int iy = ref_bin(y, P.gw[1], P.igw[1], P.gy, err);
    int iz = ref_bin(z, P.gw[2], P.igw[2], P.gz, err);
    int ip = ref_bin(ph, P.gw[3], P.igw[3], P.gphi, err);
    int it = ref_bin(th, P.gw[4], P.igw[4], P.gtheta, err);
    unsigned long long cell = (unsigned long long)((ix * P.gy + iy) * P.gz + iz);
    atomicAdd(counts + cell * (unsigned long long)P.nang + (unsigned long long)(ip * P.gtheta + it), 1u);
}

// (count / D) * V, the normalisation of sample_from and the box-volume
// rescale of do_timestep; NaN in every bin when a row was non-finite
__global__ void k_noalloc_dist(const uint32_t *__restrict__ counts, long long nbins, double den, double vol,
                               double *__restrict__ dist) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= nbins) return;
    dist[i] = counts[kErrWord] ? __longlong_as_double(0x7FF8000000000000ll) : ((double)counts[i] / den) * vol;
}

}  // namespace

extern "C" int ss_sample_distribution_noalloc(const ss_grid *grid, const ss_box *box, const double *particles,
                                              uint64_t n, double *dist, void *stream) {
    if (!grid || !box || !particles || !dist) return noalloc_fail(SS_ERR_INVALID_ARGUMENT, "null argument");
    const uint64_t lim = 1ull << 20;
    if (grid->x < 1 || grid->y < 1 || grid->z < 1 || grid->phi < 1 || grid->theta < 1 || grid->x > lim ||
        grid->y > lim || grid->z > lim || grid->phi > lim || grid->theta > lim)
        return noalloc_fail(SS_ERR_INVALID_ARGUMENT, "grid sizes must lie in [1, 2^20]");
    const uint64_t ncell = grid->x * grid->y * grid->z, nang = grid->phi * grid->theta;
    if (ncell > SS_NOALLOC_MAX_BINS || nang > SS_NOALLOC_MAX_BINS || ncell * nang > SS_NOALLOC_MAX_BINS)
        return noalloc_fail(SS_ERR_INVALID_ARGUMENT,
                            "grid has %llu x %llu bins; ss_sample_distribution_noalloc holds at most %u "
                            "(use ss_init + ss_get_distribution for larger grids)",
                            (unsigned long long)ncell, (unsigned long long)nang, (unsigned)SS_NOALLOC_MAX_BINS);
    if (!(box->x > 0.) || !(box->y > 0.) || !(box->z > 0.) || !std::isfinite(box->x) || !std::isfinite(box->y) ||
        !std::isfinite(box->z))
        return noalloc_fail(SS_ERR_INVALID_ARGUMENT, "Box size is invalid. Must be bigger than 0: (%g, %g, %g)",
                            box->x, box->y, box->z);
    if (n < 1 || n > 0xffffffffull)
        return noalloc_fail(SS_ERR_INVALID_ARGUMENT, "number_of_particles must lie in [1, 2^32-1]");

    uint32_t *counts = nullptr;
    int sms = 1;
    int rc = scratch_on_current_device(&counts, &sms);
    if (rc != SS_OK) return rc;

    DevParams P{};
    P.gx = (int)grid->x; P.gy = (int)grid->y; P.gz = (int)grid->z;
    P.gphi = (int)grid->phi; P.gtheta = (int)grid->theta;
    P.ncell = (int)ncell;
    P.nang = (int)nang;
    P.nbins = (long long)(ncell * nang);
    P.n = n;
    P.bx = box->x; P.by = box->y; P.bz = box->z;
    P.gw[0] = box->x / (double)grid->x;
    P.gw[1] = box->y / (double)grid->y;
    P.gw[2] = box->z / (double)grid->z;
    P.gw[3] = kTwoPi / (double)grid->phi;
    P.gw[4] = kPi / (double)grid->theta;
    for (int k = 0; k < 5; ++k) P.igw[k] = 1.0 / P.gw[k];
    const double den = P.gw[0] * P.gw[1] * P.gw[2] * P.gw[3] * P.gw[4] * (double)n;
    const double vol = box->x * box->y * box->z;

    cudaStream_t s = static_cast<cudaStream_t>(stream);
    long long zb = (P.nbins + 255) / 256;
    if (zb > 8ll * sms) zb = 8ll * sms;  // a grid-stride loop: eight blocks per multiprocessor suffice
    k_noalloc_zero<<<(unsigned)zb, 256, 0, s>>>(counts, P.nbins);
    k_noalloc_bin<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(particles, n, P, counts);
    k_noalloc_dist<<<(unsigned)((P.nbins + 255) / 256), 256, 0, s>>>(counts, P.nbins, den, vol, dist);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return noalloc_fail(SS_ERR_CUDA, "launch: %s", cudaGetErrorString(e));
    return SS_OK;
}
