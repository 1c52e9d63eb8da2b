// noalloc.cu -- the distribution of a particle list without any allocation.
//
// Some callers cannot call cudaMalloc or cudaFree at the point where they
// need a histogram: code that runs while a CUDA stream is being captured into
// a graph, a hook called from another library's loop where the device-wide
// synchronisation of cudaFree would stall or deadlock it, or an application
// that reserves a fixed device-memory budget at start-up and may not grow it.
// ss_sample_distribution_noalloc serves them: its only scratch is the
// file-scope device array below, of a fixed size, which every GPU that loads
// this library holds until the process exits.  It allocates nothing.
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

// scratch: one u32 count per bin, shared by every call on a device
static __device__ __align__(256) uint32_t g_noalloc_counts[SS_NOALLOC_MAX_BINS];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
uint32_t *g_counts_ptr[kMaxDevices] = {};

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

// device address of the scratch array on the current device, looked up once
// per device with that device current
int scratch_on_current_device(uint32_t **out) {
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
        g_counts_ptr[dev] = static_cast<uint32_t *>(p);
    }
    *out = g_counts_ptr[dev];
    return SS_OK;
}

__global__ void k_noalloc_zero(uint32_t *__restrict__ counts, long long nbins) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    long long stride = (long long)gridDim.x * blockDim.x;
    for (; i < nbins; i += stride) counts[i] = 0u;
}

// Particle::new (src/particle.rs:186-201) on each row, then the bin of
// Distribution::coord_to_grid, counted with an atomic add
__global__ void k_noalloc_bin(const double *__restrict__ aos, unsigned long long n, DevParams P,
                              uint32_t *__restrict__ counts) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double *p = aos + 5 * i;
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
// rescale of do_timestep
__global__ void k_noalloc_dist(const uint32_t *__restrict__ counts, long long nbins, double den, double vol,
                               double *__restrict__ dist) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= nbins) return;
    dist[i] = ((double)counts[i] / den) * vol;
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
    if (n < 1) return noalloc_fail(SS_ERR_INVALID_ARGUMENT, "n must be at least 1");

    uint32_t *counts = nullptr;
    int rc = scratch_on_current_device(&counts);
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
    if (zb > 152 * 16) zb = 152 * 16;
    k_noalloc_zero<<<(unsigned)zb, 256, 0, s>>>(counts, P.nbins);
    k_noalloc_bin<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(particles, n, P, counts);
    k_noalloc_dist<<<(unsigned)((P.nbins + 255) / 256), 256, 0, s>>>(counts, P.nbins, den, vol, dist);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return noalloc_fail(SS_ERR_CUDA, "launch: %s", cudaGetErrorString(e));
    return SS_OK;
}
