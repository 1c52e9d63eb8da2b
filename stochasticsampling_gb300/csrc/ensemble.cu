// ensemble.cu -- batched ensembles of independent 2-D simulations (ss_ens).
//
// Members differ in particle count, grid (edge, angle bins), box and
// parameters.  All members' particles live in one set of arrays and every
// stage of a step is one launch over all members:
//   contract  thread per global cell -> FP32 stress + density, FP64 sums
//   center    remove each member's per-component FP64 mean
//   cuFFT     one batched C2C per grid shape (members of a shape are
//             contiguous, so one plan of batch members x components covers
//             them), forward and inverse
//   kspace    thread per global cell (Oseen projection + screening, i k u)
//   table     thread per global cell -> FP32 row per cell
//   update    persistent kernel over (member, tile) work units
// and the whole step is captured once as a CUDA graph.  The arithmetic is
// the mixed-precision step of mixed.cu (FP32, positions accumulated in FP64,
// mean handling in FP64), with the same device functions and the same
// Philox stream per member (seed = member seed, counter = member-local
// particle index and timestep), so a member evolves exactly like a
// stand-alone SS_FLAG_MIXED context with the same parameters up to the
// round-off of the differently batched FFTs.
//
// The update's launch shape (threads per block, blocks per SM, particles per
// work unit) is chosen by an own autotuner that times the candidates on the
// ensemble's own data at first use.
#include <cufft.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <map>
#include <string>
#include <vector>

#include "../../include/ssgpu.h"
#include "kernels.cuh"
#include "mixed_device.cuh"

using namespace ss;

namespace {

struct EnsMember {
    MixedParams M;
    unsigned long long part_off;
    long long bin_off;
    long long fwd_off;  // float2 index of component 0 of this member's forward spectra
    long long inv_off;
    int cell_off;
    int kern_off;
    int lut_off;  // kEnsLut FP32 distribution values of the counts 0 .. kEnsLut - 1
    int chunk0, nchunk;  // the member's cell chunks (consecutive in the chunk list)
    float screening;
    float stepx, stepy;
};

struct WorkUnit {  // a tile of one member's particles
    unsigned long long start;
    uint32_t count;
    uint32_t member;
};

struct CellChunk {  // up to kChunkCells consecutive cells of one member
    uint32_t member;
    int cell0;  // member-local
    int count;
};

constexpr int kEnsRow = TABLE_STRIDE;  // no dipolar terms in the ensemble
constexpr int kEnsLut = 4096;          // the count -> value table of the single context
constexpr uint32_t kEnsMaxMembers = 4096;
constexpr int kEnsMaxPhi = 256;
constexpr int kChunkCells = 128;                // threads of the cell kernels
constexpr int kChunkCountBytes = 36 * 1024;     // shared-memory budget for one chunk's counts

// cells per chunk of a member with `na` angle bins (the chunk's counts fit the budget)
inline int chunk_cells(int na) { return std::min(kChunkCells, kChunkCountBytes / (4 * na)); }

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------
// Particle::new of one member's rows (the canonical quasi-2-D state: z = 0,
// theta = pi/2 are checked on the host and not stored)
__global__ void k_ens_ingest(const double *__restrict__ aos, unsigned long long start, unsigned long long n,
                             double bx, double by, double *__restrict__ x, double *__restrict__ y,
                             float *__restrict__ phi) {
    unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (k >= n) return;
    const double *p = aos + 5 * k;
    double ph = p[3], th = p[4];
    ref_ang_pbc(ph, th);
    ref_ang_pbc(ph, th);
    const unsigned long long i = start + k;
    x[i] = ref_modulo(ref_modulo(p[0], bx), bx);
    y[i] = ref_modulo(ref_modulo(p[1], by), by);
    phi[i] = (float)ph;
}

// the 2-D bin of bin_mixed (z = 0 and theta = pi/2 fall in bin 0 of their
// one-bin axes): cell = ix * gy + iy, bin = cell * gphi + iphi
__device__ __forceinline__ void bin2d(const MixedParams &M, double x, double y, float phi, int &cell, int &bin) {
    const int ix = bin_f(d2f_pos(x), M.igwf[0], M.gx), iy = bin_f(d2f_pos(y), M.igwf[1], M.gy);
    cell = ix * M.gy + iy;
    bin = cell * M.gphi + bin_f(phi, M.igwf[3], M.gphi);
}

__global__ void k_ens_bin(const WorkUnit *__restrict__ units, int nunits, const EnsMember *__restrict__ mem,
                          const double *__restrict__ x, const double *__restrict__ y, const float *__restrict__ phi,
                          uint32_t *__restrict__ counts) {
    for (int u = blockIdx.x; u < nunits; u += gridDim.x) {
        const WorkUnit w = units[u];
        const EnsMember &E = mem[w.member];
        for (uint32_t t = threadIdx.x; t < w.count; t += blockDim.x) {
            const unsigned long long i = w.start + t;
            int cell, bin;
            bin2d(E.M, x[i], y[i], phi[i], cell, bin);
            atomicAdd(counts + E.bin_off + bin, 1u);
        }
    }
}

// Angular contraction, one block per cell chunk of one member: the chunk's
// counts (contiguous) and the member's 9 x nang stress kernel are staged in
// shared memory with coalesced loads; thread c then sums its cell's row,
// visiting the angles from a = c mod nang on so that a warp's shared-memory
// reads fall in different banks.  The chunk's 9 component sums go to
// partials[chunk][9]; k_ens_means adds a member's chunks in chunk order, so
// the sums are the same bit for bit from run to run.
__global__ void __launch_bounds__(kChunkCells) k_ens_contract(const CellChunk *__restrict__ chunks,
                                                              const EnsMember *__restrict__ mem,
                                                              const uint32_t *__restrict__ counts,
                                                              const float *__restrict__ kern,
                                                              const float *__restrict__ lut,
                                                              float2 *__restrict__ fwd, float *__restrict__ diff,
                                                              double *__restrict__ partials) {
    extern __shared__ uint32_t s_counts[];
    __shared__ float s_kern[9 * kEnsMaxPhi];
    __shared__ double s_red[kChunkCells / 32][9];
    const CellChunk ch = chunks[blockIdx.x];
    const EnsMember &E = mem[ch.member];
    const int na = E.M.nang, tid = threadIdx.x;
    const uint32_t *src = counts + E.bin_off + (long long)ch.cell0 * na;
    for (int e = tid; e < ch.count * na; e += blockDim.x) s_counts[e] = src[e];
    for (int e = tid; e < 9 * na; e += blockDim.x) s_kern[e] = kern[E.kern_off + e];
    __syncthreads();
    float acc[9];
#pragma unroll
    for (int j = 0; j < 9; ++j) acc[j] = 0.f;
    const bool live = tid < ch.count;
    if (live) {
        const uint32_t *row = s_counts + tid * na;
        const float *L = lut + E.lut_off;
        float dens = 0.f;
        int a = tid % na;
        for (int i = 0; i < na; ++i) {
            const uint32_t n = row[a];
            const float f = (n < (uint32_t)kEnsLut) ? __ldg(L + n) : (float)(((double)n / E.M.dist_den) * E.M.volume);
#pragma unroll
            for (int j = 0; j < 9; ++j) acc[j] = fmaf(s_kern[j * na + a], f, acc[j]);
            dens += f;
            a = (a + 1 == na) ? 0 : a + 1;
        }
        const int nc = E.M.ncell, local = ch.cell0 + tid;
#pragma unroll
        for (int j = 0; j < 9; ++j) fwd[E.fwd_off + (long long)j * nc + local] = make_float2(acc[j] * E.M.measure, 0.f);
        diff[E.cell_off + local] = sqrtf(E.M.two_dt * (E.M.Dt + E.M.volex * (dens * E.M.dthph)));
    }
    // warp partials in FP32 (32 terms), the block's and the member's sums in
    // FP64 (the FP64 pipe is too slow for a per-thread tree)
#pragma unroll
    for (int j = 0; j < 9; ++j) {
        float v = live ? acc[j] * E.M.measure : 0.f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((tid & 31) == 0) s_red[tid >> 5][j] = (double)v;
    }
    __syncthreads();
    if (tid < 9) {
        double v = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += s_red[w][tid];
        partials[9ll * blockIdx.x + tid] = v;
    }
}

// per member and component: the sum of the member's chunk sums in chunk
// order (FP64), as the mean rounded to FP32
__global__ void k_ens_means(const EnsMember *__restrict__ mem, int nm, const double *__restrict__ partials,
                            float *__restrict__ means) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 9 * nm) return;
    const EnsMember &E = mem[i / 9];
    const int j = i % 9;
    double v = 0.0;
    for (int k = 0; k < E.nchunk; ++k) v += partials[9ll * (E.chunk0 + k) + j];
    means[i] = (float)(v / (double)E.M.ncell);
}

// subtract the means before the FP32 transform (the k_center_m of a single context)
__global__ void __launch_bounds__(kChunkCells) k_ens_center(const CellChunk *__restrict__ chunks,
                                                            const EnsMember *__restrict__ mem,
                                                            const float *__restrict__ means,
                                                            float2 *__restrict__ fwd) {
    const CellChunk ch = chunks[blockIdx.x];
    if ((int)threadIdx.x >= ch.count) return;
    const EnsMember &E = mem[ch.member];
    const int nc = E.M.ncell, local = ch.cell0 + threadIdx.x;
#pragma unroll
    for (int j = 0; j < 9; ++j) fwd[E.fwd_off + (long long)j * nc + local].x -= means[9 * ch.member + j];
}

__global__ void __launch_bounds__(kChunkCells) k_ens_kspace(const CellChunk *__restrict__ chunks,
                                                            const EnsMember *__restrict__ mem,
                                                            const float2 *__restrict__ fwd,
                                                            float2 *__restrict__ inv) {
    const CellChunk ch = chunks[blockIdx.x];
    if ((int)threadIdx.x >= ch.count) return;
    const EnsMember &E = mem[ch.member];
    const int nc = E.M.ncell, c = ch.cell0 + threadIdx.x;
    const int iy = c % E.M.gy, ix = c / E.M.gy;
    float k[3] = {kval_f(ix, E.M.gx, E.stepx), kval_f(iy, E.M.gy, E.stepy), 0.f};
    float s = k[0] * k[0] + k[1] * k[1];
    float ik2 = (c == 0) ? 0.f : 1.f / s;
    float inrm = (c == 0) ? 0.f : rsqrtf(s);
    float kn[3] = {k[0] * inrm, k[1] * inrm, 0.f};
    float2 sg[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        float2 a0 = fwd[E.fwd_off + (long long)(3 * r + 0) * nc + c];
        float2 a1 = fwd[E.fwd_off + (long long)(3 * r + 1) * nc + c];
        sg[r].x = a0.x * k[0] + a1.x * k[1];
        sg[r].y = a0.y * k[0] + a1.y * k[1];
    }
    float ksr = kn[0] * sg[0].x + kn[1] * sg[1].x + kn[2] * sg[2].x;
    float ksi = kn[0] * sg[0].y + kn[1] * sg[1].y + kn[2] * sg[2].y;
    float fac = (ik2 + E.screening) / (float)nc;
    float2 u[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        float tr = (sg[r].x - kn[r] * ksr) * fac, ti = (sg[r].y - kn[r] * ksi) * fac;
        u[r] = make_float2(-ti, tr);
        inv[E.inv_off + (long long)(9 + r) * nc + c] = u[r];
    }
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b)
            inv[E.inv_off + (long long)(3 * a + b) * nc + c] = make_float2(-(k[a] * u[b].y), k[a] * u[b].x);
}

// the per-cell row (u, W, E, diffusion length) of k_table_m, assembled in
// shared memory and written as whole rows (coalesced)
__global__ void __launch_bounds__(kChunkCells) k_ens_table(const CellChunk *__restrict__ chunks,
                                                           const EnsMember *__restrict__ mem,
                                                           const float2 *__restrict__ inv,
                                                           const float *__restrict__ diff,
                                                           float *__restrict__ table) {
    __shared__ float s_rows[kChunkCells][kEnsRow + 1];
    const CellChunk ch = chunks[blockIdx.x];
    const EnsMember &E = mem[ch.member];
    const int tid = threadIdx.x;
    if (tid < ch.count) {
        const int nc = E.M.ncell, c = ch.cell0 + tid;
        float g[9];
#pragma unroll
        for (int j = 0; j < 9; ++j) g[j] = inv[E.inv_off + (long long)j * nc + c].x;
        float *row = s_rows[tid];
#pragma unroll
        for (int r = 0; r < 3; ++r) row[T_U + r] = inv[E.inv_off + (long long)(9 + r) * nc + c].x;
        row[T_W01] = (g[1] - g[3]) * 0.5f;
        row[T_W02] = (g[2] - g[6]) * 0.5f;
        row[T_W12] = (g[5] - g[7]) * 0.5f;
        row[T_E00] = g[0];
        row[T_E01] = (g[1] + g[3]) * 0.5f;
        row[T_E02] = (g[2] + g[6]) * 0.5f;
        row[T_E11] = g[4];
        row[T_E12] = (g[5] + g[7]) * 0.5f;
        row[T_E22] = g[8];
        row[T_DIFF] = diff[E.cell_off + c];
        row[13] = row[14] = row[15] = 0.f;
    }
    __syncthreads();
    float *dst = table + (long long)(E.cell_off + ch.cell0) * kEnsRow;
    for (int e = tid; e < ch.count * kEnsRow; e += blockDim.x) dst[e] = s_rows[e / kEnsRow][e % kEnsRow];
}

// The persistent update: each block takes work units (a tile of one member's
// particles) round robin; the member's parameters are block-uniform and
// staged in shared memory.  The cell a particle sits in is recomputed from
// its position (the bin2d of the previous step's binning, so the same cell),
// which saves a stored cell key.  MINB (blocks per SM the compiler plans
// registers for) is one of the autotuner's choices.
template <int MINB>
__global__ void __launch_bounds__(512, MINB) k_ens_update(const WorkUnit *__restrict__ units, int nunits,
                                                          const EnsMember *__restrict__ mem,
                                                          double *__restrict__ x, double *__restrict__ y,
                                                          float *__restrict__ phi, const float *__restrict__ table,
                                                          const unsigned long long *__restrict__ d_step,
                                                          uint32_t *__restrict__ counts_next,
                                                          const uint32_t *__restrict__ pid) {
    __shared__ EnsMember E;
    const unsigned long long t = *d_step;
    for (int u = blockIdx.x; u < nunits; u += gridDim.x) {
        const WorkUnit w = units[u];
        __syncthreads();
        if (threadIdx.x == 0) E = mem[w.member];
        __syncthreads();
        const MixedParams &M = E.M;
        for (uint32_t k = threadIdx.x; k < w.count; k += blockDim.x) {
            // the member's parameters are re-read from shared memory in every
            // iteration instead of being held in registers across the loop
            asm volatile("" ::: "memory");
            const unsigned long long i = w.start + k;
            double px = x[i], py = y[i];
            float pph = phi[i], pth = 1.57079632679489661923f;
            const int cx = bin_f(d2f_pos(px), M.igwf[0], M.gx), cy = bin_f(d2f_pos(py), M.igwf[1], M.gy);
            TableFieldsF F(table + (long long)(E.cell_off + cx * M.gy + cy) * kEnsRow);
            float xi[3], ca, sa, rot;
            philox_noise_f<true>(M.seed, pid[i], t, M.sigma_rot, xi, ca, sa, rot);  // the caller's index in the member
            float st[3];
            langevin_mixed<true>(pph, pth, st, F, xi, ca, sa, rot, M);
            px = advance64(px, st[0], M.bx);
            py = advance64(py, st[1], M.by);
            int cell, bin;
            bin2d(M, px, py, pph, cell, bin);
            atomicAdd(counts_next + E.bin_off + bin, 1u);
            x[i] = px;
            y[i] = py;
            phi[i] = pph;
        }
    }
}

using UpdateKernel = void (*)(const WorkUnit *, int, const EnsMember *, double *, double *, float *, const float *,
                              const unsigned long long *, uint32_t *, const uint32_t *);
constexpr int kUpdateVariants = 3;
const UpdateKernel kUpdate[kUpdateVariants] = {k_ens_update<1>, k_ens_update<2>, k_ens_update<3>};

__global__ void k_ens_step_inc(unsigned long long *d_step) { *d_step += 1ull; }

// member rows back in the caller's order (pid: the caller's index in the member)
__global__ void k_ens_egest(unsigned long long start, unsigned long long n, const double *__restrict__ x,
                            const double *__restrict__ y, const float *__restrict__ phi,
                            const uint32_t *__restrict__ pid, double *__restrict__ aos) {
    unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (k >= n) return;
    unsigned long long i = start + k;
    double *p = aos + 5 * (unsigned long long)pid[i];
    p[0] = x[i]; p[1] = y[i]; p[2] = 0.0; p[3] = (double)phi[i]; p[4] = 1.5707963267948966;
}

__global__ void k_ens_real(const float2 *__restrict__ src, long long count, double *__restrict__ dst) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < count) dst[i] = (double)src[i].x;
}

}  // namespace

// ---------------------------------------------------------------------------
// host object
// ---------------------------------------------------------------------------
struct ss_ens {
    uint32_t nm = 0;
    std::vector<EnsMember> mem;
    struct Group {
        int gx, gy;
        std::vector<uint32_t> members;
        long long fwd_off, inv_off;
        cufftHandle fwd_plan = 0, inv_plan = 0;
    };
    std::vector<Group> groups;
    unsigned long long ntot = 0;
    int total_cells = 0;
    long long total_bins = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int device = 0, sms = 0;
    bool initialized = false;
    uint64_t timestep = 0;
    int ccur = 0;

    EnsMember *d_mem = nullptr;
    WorkUnit *d_units = nullptr;
    int nunits = 0;
    int variant = 1, threads = 256, blocks_per_sm = 4, unit = 16384;  // the update's launch shape
    bool tuned = false;
    CellChunk *d_chunks = nullptr;
    int nchunks = 0;
    size_t chunk_smem = 0;  // dynamic shared memory of k_ens_contract
    double *x = nullptr, *y = nullptr, *staging = nullptr, *realbuf = nullptr;
    // a member's rows in cell order at init (locality of the update), with each
    // particle's index in the member's caller order
    double *staging_sorted = nullptr;
    uint32_t *pid = nullptr, *cellkey = nullptr, *cellcount = nullptr, *cursor = nullptr;
    float *phi = nullptr;
    uint32_t *counts[2] = {};
    float2 *fwd = nullptr, *inv = nullptr;
    float *table = nullptr, *kern = nullptr, *lut = nullptr, *diff = nullptr, *means = nullptr;
    double *sums = nullptr;  // per cell chunk, its 9 component sums
    unsigned long long *d_step = nullptr;
    cudaGraphExec_t graph[2] = {};
    uint64_t launches = 0, step_launches = 0;
    std::string err;
};

namespace {

int efail(ss_ens *e, int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (e) e->err = buf;
    record_error(buf);
    return code;
}

#define ECK(call)                                                                                       \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess) return efail(e, SS_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_));   \
    } while (0)
#define ECKF(call)                                                                                       \
    do {                                                                                                 \
        cufftResult r_ = (call);                                                                         \
        if (r_ != CUFFT_SUCCESS) return efail(e, SS_ERR_CUFFT, "%s: cufft error %d", #call, (int)r_);   \
    } while (0)
#define ECKR(expr)                    \
    do {                              \
        int rc_ = (expr);             \
        if (rc_ != SS_OK) return rc_; \
    } while (0)

int build_units(ss_ens *e, int unit) {
    std::vector<WorkUnit> u;
    for (uint32_t m = 0; m < e->nm; ++m) {
        unsigned long long n = e->mem[m].M.n, off = e->mem[m].part_off;
        for (unsigned long long s = 0; s < n; s += (unsigned long long)unit)
            u.push_back({off + s, (uint32_t)std::min<unsigned long long>((unsigned long long)unit, n - s), m});
    }
    cudaFree(e->d_units);
    e->d_units = nullptr;
    ECK(cudaMalloc((void **)&e->d_units, std::max<size_t>(1, u.size()) * sizeof(WorkUnit)));
    ECK(cudaMemcpyAsync(e->d_units, u.data(), u.size() * sizeof(WorkUnit), cudaMemcpyHostToDevice, e->stream));
    ECK(cudaStreamSynchronize(e->stream));
    e->nunits = (int)u.size();
    e->unit = unit;
    return SS_OK;
}

unsigned nb(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

// the field solve of one step: histogram counts[ccur] -> table
int enqueue_solve(ss_ens *e, int ccur, uint64_t *nl) {
    cudaStream_t s = e->stream;
    const unsigned nc = (unsigned)e->nchunks;
    k_ens_contract<<<nc, kChunkCells, e->chunk_smem, s>>>(e->d_chunks, e->d_mem, e->counts[ccur], e->kern, e->lut,
                                                           e->fwd, e->diff, e->sums);
    k_ens_means<<<nb(9ll * e->nm, 128), 128, 0, s>>>(e->d_mem, (int)e->nm, e->sums, e->means);
    k_ens_center<<<nc, kChunkCells, 0, s>>>(e->d_chunks, e->d_mem, e->means, e->fwd);
    for (auto &g : e->groups)
        ECKF(cufftExecC2C(g.fwd_plan, reinterpret_cast<cufftComplex *>(e->fwd + g.fwd_off),
                          reinterpret_cast<cufftComplex *>(e->fwd + g.fwd_off), CUFFT_FORWARD));
    k_ens_kspace<<<nc, kChunkCells, 0, s>>>(e->d_chunks, e->d_mem, e->fwd, e->inv);
    for (auto &g : e->groups)
        ECKF(cufftExecC2C(g.inv_plan, reinterpret_cast<cufftComplex *>(e->inv + g.inv_off),
                          reinterpret_cast<cufftComplex *>(e->inv + g.inv_off), CUFFT_INVERSE));
    k_ens_table<<<nc, kChunkCells, 0, s>>>(e->d_chunks, e->d_mem, e->inv, e->diff, e->table);
    *nl += 5;
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return efail(e, SS_ERR_CUDA, "ensemble solve launch: %s", cudaGetErrorString(err));
    return SS_OK;
}

void launch_update(ss_ens *e, int variant, int threads, int bps, double *x, double *y, float *phi,
                   uint32_t *counts_next) {
    kUpdate[variant]<<<(unsigned)(e->sms * bps), threads, 0, e->stream>>>(e->d_units, e->nunits, e->d_mem, x, y, phi,
                                                                         e->table, e->d_step, counts_next, e->pid);
}

// one do_timestep of every member: solve from counts[ccur], move the
// particles, bin them into counts[1 - ccur]
int enqueue_step(ss_ens *e, int ccur, uint64_t *nl) {
    cudaStream_t s = e->stream;
    ECKR(enqueue_solve(e, ccur, nl));
    ECK(cudaMemsetAsync(e->counts[1 - ccur], 0, (size_t)e->total_bins * sizeof(uint32_t), s));
    launch_update(e, e->variant, e->threads, e->blocks_per_sm, e->x, e->y, e->phi, e->counts[1 - ccur]);
    k_ens_step_inc<<<1, 1, 0, s>>>(e->d_step);
    *nl += 2;
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return efail(e, SS_ERR_CUDA, "ensemble update launch: %s", cudaGetErrorString(err));
    return SS_OK;
}

// Autotuner for the persistent update: every candidate (register plan of
// 1, 2 or 3 blocks per SM; threads per block; resident blocks per SM;
// particles per work unit) runs the update on a scratch copy of the
// ensemble's particles through the fields of the current histogram; the
// fastest median of three wins.  The candidates do not change the
// ensemble's state.
struct TuneScratch {
    double *x = nullptr, *y = nullptr;
    float *phi = nullptr;
    uint32_t *counts = nullptr;
    cudaEvent_t a = nullptr, b = nullptr;
    ~TuneScratch() {
        cudaFree(x); cudaFree(y); cudaFree(phi); cudaFree(counts);
        if (a) cudaEventDestroy(a);
        if (b) cudaEventDestroy(b);
    }
};

int autotune(ss_ens *e) {
    const int th[] = {128, 256, 512};
    const int bps[] = {2, 4, 8};
    const int un[] = {4096, 16384, 65536};
    // the captured steps hold the work-unit list, which the candidates rebuild
    for (auto &g : e->graph)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
    TuneScratch S;
    const size_t N = (size_t)e->ntot;
    ECK(cudaMalloc((void **)&S.x, N * sizeof(double)));
    ECK(cudaMalloc((void **)&S.y, N * sizeof(double)));
    ECK(cudaMalloc((void **)&S.phi, N * sizeof(float)));
    ECK(cudaMalloc((void **)&S.counts, (size_t)e->total_bins * sizeof(uint32_t)));
    ECK(cudaEventCreate(&S.a));
    ECK(cudaEventCreate(&S.b));
    uint64_t nl = 0;
    ECKR(enqueue_solve(e, e->ccur, &nl));
    e->launches += nl;
    float best = 1e30f;
    int bv = e->variant, bt = e->threads, bb = e->blocks_per_sm, bu = e->unit;
    for (int unit : un) {
        ECKR(build_units(e, unit));
        for (int v = 0; v < kUpdateVariants; ++v)
            for (int t : th)
                for (int k : bps) {
                    float ms[3];
                    for (int r = 0; r < 3; ++r) {
                        ECK(cudaMemcpyAsync(S.x, e->x, N * sizeof(double), cudaMemcpyDeviceToDevice, e->stream));
                        ECK(cudaMemcpyAsync(S.y, e->y, N * sizeof(double), cudaMemcpyDeviceToDevice, e->stream));
                        ECK(cudaMemcpyAsync(S.phi, e->phi, N * sizeof(float), cudaMemcpyDeviceToDevice, e->stream));
                        ECK(cudaMemsetAsync(S.counts, 0, (size_t)e->total_bins * sizeof(uint32_t), e->stream));
                        ECK(cudaEventRecord(S.a, e->stream));
                        launch_update(e, v, t, k, S.x, S.y, S.phi, S.counts);
                        cudaError_t le = cudaGetLastError();
                        if (le == cudaErrorLaunchOutOfResources || le == cudaErrorInvalidConfiguration) {
                            ms[r] = 1e30f;  // shape not launchable on this device: never chosen
                            continue;
                        }
                        if (le != cudaSuccess) return efail(e, SS_ERR_CUDA, "autotune: %s", cudaGetErrorString(le));
                        e->launches += 1;
                        ECK(cudaEventRecord(S.b, e->stream));
                        ECK(cudaEventSynchronize(S.b));
                        ECK(cudaEventElapsedTime(&ms[r], S.a, S.b));
                    }
                    std::sort(ms, ms + 3);
                    if (ms[1] < best) {
                        best = ms[1];
                        bv = v;
                        bt = t;
                        bb = k;
                        bu = unit;
                    }
                }
    }
    e->variant = bv;
    e->threads = bt;
    e->blocks_per_sm = bb;
    ECKR(build_units(e, bu));
    e->tuned = true;
    return SS_OK;
}

void destroy(ss_ens *e) {
    if (!e) return;
    cudaSetDevice(e->device);
    if (e->stream) cudaStreamSynchronize(e->stream);
    for (auto &g : e->groups) {
        if (g.fwd_plan) cufftDestroy(g.fwd_plan);
        if (g.inv_plan) cufftDestroy(g.inv_plan);
    }
    for (auto &g : e->graph)
        if (g) cudaGraphExecDestroy(g);
    cudaFree(e->d_mem); cudaFree(e->d_units); cudaFree(e->d_chunks); cudaFree(e->x); cudaFree(e->y);
    cudaFree(e->staging); cudaFree(e->staging_sorted); cudaFree(e->pid); cudaFree(e->cellkey);
    cudaFree(e->cellcount); cudaFree(e->cursor); cudaFree(e->realbuf); cudaFree(e->phi); cudaFree(e->diff); cudaFree(e->means);
    cudaFree(e->counts[0]);
    cudaFree(e->counts[1]); cudaFree(e->fwd); cudaFree(e->inv); cudaFree(e->table); cudaFree(e->kern); cudaFree(e->lut);
    cudaFree(e->sums); cudaFree(e->d_step);
    if (e->own_stream && e->stream) cudaStreamDestroy(e->stream);
    delete e;
}

}  // namespace

extern "C" {

int ss_ensemble_create(const ss_grid *grids, const ss_box *boxes, const ss_params *params, uint32_t count,
                       uint32_t flags, void *stream, ss_ens **out) {
    if (!grids || !boxes || !params || !out || count == 0)
        return efail(nullptr, SS_ERR_INVALID_ARGUMENT, "ss_ensemble_create: null argument or no member");
    *out = nullptr;
    if (count > kEnsMaxMembers)
        return efail(nullptr, SS_ERR_INVALID_ARGUMENT, "ss_ensemble_create: at most %u members", kEnsMaxMembers);
    if (!(flags & SS_FLAG_QUASI2D) || (flags & ~(uint32_t)(SS_FLAG_QUASI2D | SS_FLAG_MIXED)))
        return efail(nullptr, SS_ERR_INVALID_ARGUMENT,
                     "ss_ensemble_create: ensembles are quasi-2-D and mixed precision (flags QUASI2D [| MIXED])");
    unsigned long long part = 0;
    long long bins = 0, cells = 0;
    for (uint32_t m = 0; m < count; ++m) {
        const ss_grid &g = grids[m];
        const ss_box &b = boxes[m];
        const ss_params &p = params[m];
        if (g.x < 2 || g.y < 2 || g.z != 1 || g.theta != 1 || g.phi < 1 || g.x > 4096 || g.y > 4096 ||
            g.phi > (uint64_t)kEnsMaxPhi)
            return efail(nullptr, SS_ERR_INVALID_ARGUMENT,
                         "member %u: grid must be quasi-2-D (z = theta = 1, 2 <= x, y <= 4096, 1 <= phi <= %d)", m,
                         kEnsMaxPhi);
        if (!(b.x > 0) || !(b.y > 0) || !(b.z > 0) || !std::isfinite(b.x) || !std::isfinite(b.y) ||
            !std::isfinite(b.z))
            return efail(nullptr, SS_ERR_INVALID_ARGUMENT, "member %u: box sizes must be positive and finite", m);
        if (p.number_of_particles < 1 || p.number_of_particles > 0xffffffffull)
            return efail(nullptr, SS_ERR_INVALID_ARGUMENT, "member %u: 1 <= particles < 2^32", m);
        if (p.magnetic_dipole_dipole != 0.0 || p.magnetic_drag != 0.0)
            return efail(nullptr, SS_ERR_INVALID_ARGUMENT,
                         "member %u: ensembles have no dipolar coupling (magnetic_dipole_dipole = magnetic_drag = 0)",
                         m);
        const double pv[] = {p.timestep, p.trans_diffusion, p.rot_diffusion, p.stress_active, p.stress_magnetic,
                             p.shape, p.magnetic_reorientation, p.volume_exclusion, p.hydro_screening};
        for (double v : pv)
            if (!std::isfinite(v)) return efail(nullptr, SS_ERR_INVALID_ARGUMENT, "member %u: non-finite parameter", m);
        part += p.number_of_particles;
        cells += (long long)(g.x * g.y);
        bins += (long long)(g.x * g.y * g.phi);
    }
    if (cells > (1ll << 28) || bins > (1ll << 31) || part > (1ull << 36))
        return efail(nullptr, SS_ERR_INVALID_ARGUMENT,
                     "ss_ensemble_create: ensemble too large (cells <= 2^28, bins <= 2^31, particles <= 2^36)");

    ss_ens *e = new ss_ens();
    e->nm = count;
    e->mem.resize(count);
    e->ntot = part;
    e->total_cells = (int)cells;
    e->total_bins = bins;
    std::map<std::pair<int, int>, int> gid;
    part = 0;
    bins = 0;
    cells = 0;
    int max_cell = 0;
    unsigned long long max_n = 0;
    for (uint32_t m = 0; m < count; ++m) {
        const ss_grid &g = grids[m];
        const ss_box &b = boxes[m];
        const ss_params &p = params[m];
        auto key = std::make_pair((int)g.x, (int)g.y);
        if (!gid.count(key)) {
            gid[key] = (int)e->groups.size();
            e->groups.push_back({(int)g.x, (int)g.y, {}, 0, 0});
        }
        e->groups[gid[key]].members.push_back(m);
        // the parameters of a single SS_FLAG_MIXED | SS_FLAG_QUASI2D context (ssgpu.cu)
        EnsMember &E = e->mem[m];
        MixedParams &M = E.M;
        M.gx = (int)g.x; M.gy = (int)g.y; M.gz = 1; M.gphi = (int)g.phi; M.gtheta = 1;
        M.ncell = (int)(g.x * g.y);
        M.nang = (int)g.phi;
        M.n = p.number_of_particles;
        M.bx = b.x; M.by = b.y; M.bz = b.z;
        M.bx2 = 2.0 * b.x; M.by2 = 2.0 * b.y; M.bz2 = 2.0 * b.z;
        const double gw[5] = {b.x / (double)g.x, b.y / (double)g.y, b.z / 1.0, kTwoPi / (double)g.phi, kPi / 1.0};
        for (int k = 0; k < 5; ++k) M.igwf[k] = (float)(1.0 / gw[k]);
        const double L[3] = {b.x, b.y, b.z};
        for (int k = 0; k < 3; ++k) {
            M.gwf[k] = (float)gw[k];
            M.s32[k] = (float)(0x1p32 / L[k]);
            M.unit[k] = L[k] * 0x1p-64;
        }
        M.dist_den = gw[0] * gw[1] * gw[2] * gw[3] * gw[4] * (double)M.n;
        M.volume = b.x * b.y * b.z;
        M.measure = (float)(gw[3] * gw[4]);
        M.dthph = (float)(gw[4] * gw[3]);
        M.two_dt = (float)(2.0 * p.timestep);
        M.Dt = (float)p.trans_diffusion;
        M.volex = (float)p.volume_exclusion;
        M.dt = (float)p.timestep;
        M.drag = 0.f;
        M.reorient = (float)p.magnetic_reorientation;
        M.shape = (float)p.shape;
        M.mdd = 0.f;
        M.sigma_rot = (float)std::sqrt(2. * p.rot_diffusion * p.timestep);
        M.seed = p.seed;
        uint32_t mask = M_ALL & ~(uint32_t)(M_MDD_FORCE | M_MDD_ROTATION);
        if (p.magnetic_reorientation == 0.0) mask &= ~(uint32_t)M_EXTERNAL_FIELD;
        if (p.shape == 0.0) mask &= ~(uint32_t)M_JEFFREY_STRAIN;
        M.mask = mask;
        E.part_off = part;
        E.bin_off = bins;
        E.cell_off = (int)cells;
        E.lut_off = (int)m * kEnsLut;
        E.screening = (float)p.hydro_screening;
        E.stepx = (float)(kTwoPi / b.x);
        E.stepy = (float)(kTwoPi / b.y);
        part += M.n;
        bins += (long long)M.ncell * M.nang;
        cells += M.ncell;
        max_cell = std::max(max_cell, M.ncell);
        max_n = std::max(max_n, M.n);
    }
    // spectra: the members of one grid shape contiguous, one batched plan per shape
    long long fo = 0, io = 0;
    for (auto &g : e->groups) {
        g.fwd_off = fo;
        g.inv_off = io;
        for (uint32_t m : g.members) {
            e->mem[m].fwd_off = fo;
            e->mem[m].inv_off = io;
            fo += 9ll * e->mem[m].M.ncell;
            io += 12ll * e->mem[m].M.ncell;
        }
    }
    // angle kernels (FP64 -> FP32, the first 9 components) and count tables
    std::vector<double> K;
    std::vector<float> kern, lut((size_t)count * kEnsLut);
    for (uint32_t m = 0; m < count; ++m) {
        build_angle_kernels(grids[m], params[m], K);
        e->mem[m].kern_off = (int)kern.size();
        kern.insert(kern.end(), K.begin(), K.begin() + 9 * (size_t)e->mem[m].M.nang);
        for (int i = 0; i < kEnsLut; ++i)
            lut[(size_t)m * kEnsLut + i] = (float)(((double)i / e->mem[m].M.dist_den) * e->mem[m].M.volume);
    }
    // cell chunks: member-aligned blocks of the cell kernels
    std::vector<CellChunk> chunks;
    for (uint32_t m = 0; m < count; ++m) {
        const int nc = e->mem[m].M.ncell, per = chunk_cells(e->mem[m].M.nang);
        e->mem[m].chunk0 = (int)chunks.size();
        for (int c0 = 0; c0 < nc; c0 += per) chunks.push_back({m, c0, std::min(per, nc - c0)});
        e->mem[m].nchunk = (int)chunks.size() - e->mem[m].chunk0;
        e->chunk_smem = std::max(e->chunk_smem, (size_t)per * e->mem[m].M.nang * sizeof(uint32_t));
    }
    e->nchunks = (int)chunks.size();

    cudaError_t err = cudaGetDevice(&e->device);
    if (err == cudaSuccess) err = cudaDeviceGetAttribute(&e->sms, cudaDevAttrMultiProcessorCount, e->device);
    if (err == cudaSuccess) {
        if (stream) {
            e->stream = (cudaStream_t)stream;
        } else {
            err = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking);
            e->own_stream = err == cudaSuccess;
        }
    }
    const size_t N = (size_t)e->ntot;
    auto A = [&](void **p, size_t bytes) {
        if (err == cudaSuccess) err = cudaMalloc(p, std::max<size_t>(bytes, 16));
    };
    A((void **)&e->d_mem, count * sizeof(EnsMember));
    A((void **)&e->d_chunks, chunks.size() * sizeof(CellChunk));
    A((void **)&e->diff, (size_t)e->total_cells * sizeof(float));
    A((void **)&e->means, 9ull * count * sizeof(float));
    A((void **)&e->x, N * sizeof(double));
    A((void **)&e->y, N * sizeof(double));
    A((void **)&e->phi, N * sizeof(float));
    A((void **)&e->counts[0], (size_t)e->total_bins * sizeof(uint32_t));
    A((void **)&e->counts[1], (size_t)e->total_bins * sizeof(uint32_t));
    A((void **)&e->fwd, (size_t)fo * sizeof(float2));
    A((void **)&e->inv, (size_t)io * sizeof(float2));
    A((void **)&e->table, (size_t)e->total_cells * kEnsRow * sizeof(float));
    A((void **)&e->kern, kern.size() * sizeof(float));
    A((void **)&e->lut, lut.size() * sizeof(float));
    A((void **)&e->sums, 9ull * chunks.size() * sizeof(double));
    A((void **)&e->d_step, sizeof(unsigned long long));
    A((void **)&e->realbuf, 3ull * max_cell * sizeof(double));
    A((void **)&e->staging, 5ull * max_n * sizeof(double));
    A((void **)&e->staging_sorted, 5ull * max_n * sizeof(double));
    A((void **)&e->pid, N * sizeof(uint32_t));
    A((void **)&e->cellkey, max_n * sizeof(uint32_t));
    A((void **)&e->cellcount, (size_t)max_cell * sizeof(uint32_t));
    A((void **)&e->cursor, (size_t)max_cell * sizeof(uint32_t));
    // every copy on the ensemble's stream (a non-blocking stream does not
    // order itself after the legacy stream of a plain cudaMemcpy)
    const cudaStream_t st = e->stream;
    if (err == cudaSuccess)
        err = cudaMemcpyAsync(e->d_mem, e->mem.data(), count * sizeof(EnsMember), cudaMemcpyHostToDevice, st);
    if (err == cudaSuccess)
        err = cudaMemcpyAsync(e->d_chunks, chunks.data(), chunks.size() * sizeof(CellChunk), cudaMemcpyHostToDevice,
                              st);
    if (err == cudaSuccess)
        err = cudaMemcpyAsync(e->kern, kern.data(), kern.size() * sizeof(float), cudaMemcpyHostToDevice, st);
    if (err == cudaSuccess)
        err = cudaMemcpyAsync(e->lut, lut.data(), lut.size() * sizeof(float), cudaMemcpyHostToDevice, st);
    if (err == cudaSuccess) err = cudaMemsetAsync(e->inv, 0, (size_t)io * sizeof(float2), st);
    if (err == cudaSuccess) err = cudaMemsetAsync(e->table, 0, (size_t)e->total_cells * kEnsRow * sizeof(float), st);
    if (err == cudaSuccess) err = cudaMemsetAsync(e->d_step, 0, sizeof(unsigned long long), st);
    if (err == cudaSuccess) err = cudaStreamSynchronize(st);
    if (err != cudaSuccess) {
        std::string msg = cudaGetErrorString(err);
        destroy(e);
        return efail(nullptr, SS_ERR_CUDA, "ss_ensemble_create: %s", msg.c_str());
    }
    for (auto &g : e->groups) {
        int n[2] = {g.gx, g.gy};
        const int nc = g.gx * g.gy, nmem = (int)g.members.size();
        cufftResult r = cufftPlanMany(&g.fwd_plan, 2, n, nullptr, 1, nc, nullptr, 1, nc, CUFFT_C2C, 9 * nmem);
        if (r == CUFFT_SUCCESS) r = cufftPlanMany(&g.inv_plan, 2, n, nullptr, 1, nc, nullptr, 1, nc, CUFFT_C2C, 12 * nmem);
        if (r == CUFFT_SUCCESS) r = cufftSetStream(g.fwd_plan, e->stream);
        if (r == CUFFT_SUCCESS) r = cufftSetStream(g.inv_plan, e->stream);
        if (r != CUFFT_SUCCESS) {
            destroy(e);
            return efail(nullptr, SS_ERR_CUFFT, "ss_ensemble_create: cufft plan error %d", (int)r);
        }
    }
    int rc = build_units(e, e->unit);
    if (rc != SS_OK) {
        std::string msg = e->err;
        destroy(e);
        return efail(nullptr, rc, "%s", msg.c_str());
    }
    *out = e;
    return SS_OK;
}

int ss_ensemble_destroy(ss_ens *e) {
    destroy(e);
    return SS_OK;
}

int ss_ensemble_init(ss_ens *e, const double *particles, uint64_t total) {
    if (!e || !particles) return efail(e, SS_ERR_INVALID_ARGUMENT, "null argument");
    if (total != e->ntot)
        return efail(e, SS_ERR_PARTICLE_COUNT, "expected %llu particles (the members' sum), got %llu",
                     (unsigned long long)e->ntot, (unsigned long long)total);
    for (uint64_t i = 0; i < total; ++i) {
        const double *p = particles + 5 * i;
        for (int k = 0; k < 5; ++k)
            if (!std::isfinite(p[k]))
                return efail(e, SS_ERR_INVALID_ARGUMENT, "particle %llu has a non-finite coordinate",
                             (unsigned long long)i);
        if (p[2] != 0.0 || p[4] != kPiHalf)
            return efail(e, SS_ERR_INVALID_ARGUMENT, "particle %llu: ensemble members are quasi-2-D (z = 0, theta = pi/2)",
                         (unsigned long long)i);
    }
    ECK(cudaSetDevice(e->device));
    for (uint32_t m = 0; m < e->nm; ++m) {
        const EnsMember &E = e->mem[m];
        ECK(cudaMemcpyAsync(e->staging, particles + 5 * E.part_off, 5 * E.M.n * sizeof(double),
                            cudaMemcpyHostToDevice, e->stream));
        // the member's rows in cell order, their caller indices into pid
        DevParams P{};
        P.gx = E.M.gx; P.gy = E.M.gy; P.gz = 1; P.ncell = E.M.gx * E.M.gy;
        P.bx = E.M.bx; P.by = E.M.by; P.bz = 1.0;
        P.igwf[0] = E.M.igwf[0]; P.igwf[1] = E.M.igwf[1]; P.igwf[2] = 1.0f;
        launch_sort_rows(e->stream, e->staging, E.M.n, P, e->cellkey, e->cellcount, e->cursor, e->staging_sorted,
                         e->pid + E.part_off);
        k_ens_ingest<<<nb((long long)E.M.n, 256), 256, 0, e->stream>>>(e->staging_sorted, E.part_off, E.M.n, E.M.bx,
                                                                        E.M.by, e->x, e->y, e->phi);
        ECK(cudaGetLastError());
    }
    ECK(cudaMemsetAsync(e->counts[0], 0, (size_t)e->total_bins * sizeof(uint32_t), e->stream));
    k_ens_bin<<<(unsigned)(e->sms * 4), 256, 0, e->stream>>>(e->d_units, e->nunits, e->d_mem, e->x, e->y, e->phi,
                                                              e->counts[0]);
    ECK(cudaGetLastError());
    e->launches += 5 * e->nm + 1;
    ECK(cudaMemsetAsync(e->d_step, 0, sizeof(unsigned long long), e->stream));
    ECK(cudaStreamSynchronize(e->stream));
    e->ccur = 0;
    e->timestep = 0;
    e->initialized = true;
    return SS_OK;
}

int ss_ensemble_autotune(ss_ens *e, uint32_t *config) {
    if (!e) return efail(nullptr, SS_ERR_INVALID_ARGUMENT, "null ensemble");
    if (!e->initialized) return efail(e, SS_ERR_STATE, "ss_ensemble_autotune before ss_ensemble_init");
    ECK(cudaSetDevice(e->device));
    ECKR(autotune(e));
    if (config) {
        config[0] = (uint32_t)e->threads;
        config[1] = (uint32_t)e->blocks_per_sm;
        config[2] = (uint32_t)e->unit;
        config[3] = (uint32_t)e->variant + 1;
    }
    return SS_OK;
}

int ss_ensemble_set_config(ss_ens *e, const uint32_t *config) {
    if (!e || !config) return efail(e, SS_ERR_INVALID_ARGUMENT, "null argument");
    const uint32_t t = config[0], k = config[1], u = config[2], v = config[3];
    if (t == 0 || t > 512 || t % 32 != 0 || k < 1 || k > 32 || u < 32 || u > (1u << 24) || v < 1 ||
        v > (uint32_t)kUpdateVariants)
        return efail(e, SS_ERR_INVALID_ARGUMENT,
                     "update config: threads a multiple of 32 in [32, 512], blocks per SM in [1, 32], "
                     "particles per unit in [32, 2^24], register plan in [1, %d]",
                     kUpdateVariants);
    ECK(cudaSetDevice(e->device));
    for (auto &g : e->graph)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
    e->threads = (int)t;
    e->blocks_per_sm = (int)k;
    e->variant = (int)v - 1;
    ECKR(build_units(e, (int)u));
    e->tuned = true;
    return SS_OK;
}

int ss_ensemble_run(ss_ens *e, uint64_t steps) {
    if (!e) return efail(nullptr, SS_ERR_INVALID_ARGUMENT, "null ensemble");
    if (!e->initialized) return efail(e, SS_ERR_STATE, "ss_ensemble_run before ss_ensemble_init");
    ECK(cudaSetDevice(e->device));
    if (!e->tuned) ECKR(autotune(e));
    for (uint64_t k = 0; k < steps; ++k) {
        cudaGraphExec_t &g = e->graph[e->ccur];
        if (!g) {
            cudaGraph_t graph;
            uint64_t nl = 0;
            ECK(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
            int rc = enqueue_step(e, e->ccur, &nl);
            cudaError_t err = cudaStreamEndCapture(e->stream, &graph);
            if (rc != SS_OK) {
                if (err == cudaSuccess) cudaGraphDestroy(graph);
                return rc;
            }
            if (err != cudaSuccess) return efail(e, SS_ERR_CUDA, "graph capture: %s", cudaGetErrorString(err));
            err = cudaGraphInstantiate(&g, graph, 0);
            cudaGraphDestroy(graph);
            if (err != cudaSuccess) return efail(e, SS_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(err));
            e->step_launches = nl;
        }
        ECK(cudaGraphLaunch(g, e->stream));
        e->launches += e->step_launches;
        e->ccur ^= 1;
        e->timestep += 1;
    }
    return SS_OK;
}

int ss_ensemble_synchronize(ss_ens *e) {
    if (!e) return efail(nullptr, SS_ERR_INVALID_ARGUMENT, "null ensemble");
    ECK(cudaStreamSynchronize(e->stream));
    return SS_OK;
}

int ss_ensemble_get_particles(ss_ens *e, uint32_t member, double *out) {
    if (!e || !out || member >= e->nm) return efail(e, SS_ERR_INVALID_ARGUMENT, "bad member or null argument");
    ECK(cudaSetDevice(e->device));
    const EnsMember &E = e->mem[member];
    k_ens_egest<<<nb((long long)E.M.n, 256), 256, 0, e->stream>>>(E.part_off, E.M.n, e->x, e->y, e->phi, e->pid,
                                                                    e->staging);
    ECK(cudaGetLastError());
    ECK(cudaMemcpyAsync(out, e->staging, 5 * E.M.n * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
    ECK(cudaStreamSynchronize(e->stream));
    return SS_OK;
}

int ss_ensemble_get_counts(ss_ens *e, uint32_t member, uint32_t *out) {
    if (!e || !out || member >= e->nm) return efail(e, SS_ERR_INVALID_ARGUMENT, "bad member or null argument");
    ECK(cudaSetDevice(e->device));
    const EnsMember &E = e->mem[member];
    // the histogram the last step solved from (after init: the initial one)
    const int idx = e->timestep == 0 ? e->ccur : 1 - e->ccur;
    ECK(cudaMemcpyAsync(out, e->counts[idx] + E.bin_off, (size_t)E.M.ncell * E.M.nang * sizeof(uint32_t),
                        cudaMemcpyDeviceToHost, e->stream));
    ECK(cudaStreamSynchronize(e->stream));
    return SS_OK;
}

int ss_ensemble_get_flow_field(ss_ens *e, uint32_t member, double *out) {
    if (!e || !out || member >= e->nm) return efail(e, SS_ERR_INVALID_ARGUMENT, "bad member or null argument");
    ECK(cudaSetDevice(e->device));
    const EnsMember &E = e->mem[member];
    const long long cnt = 3ll * E.M.ncell;
    k_ens_real<<<nb(cnt, 256), 256, 0, e->stream>>>(e->inv + E.inv_off + 9ll * E.M.ncell, cnt, e->realbuf);
    ECK(cudaGetLastError());
    ECK(cudaMemcpyAsync(out, e->realbuf, cnt * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
    ECK(cudaStreamSynchronize(e->stream));
    return SS_OK;
}

int ss_ensemble_info(ss_ens *e, uint64_t *particles, uint32_t *groups, uint64_t *launches) {
    if (!e) return efail(nullptr, SS_ERR_INVALID_ARGUMENT, "null ensemble");
    if (particles) *particles = e->ntot;
    if (groups) *groups = (uint32_t)e->groups.size();
    if (launches) *launches = e->launches;
    return SS_OK;
}

}  // extern "C"
