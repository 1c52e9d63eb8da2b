// contract.cu -- the angular contraction of the histogram for the FP64 and the
// FP32 mixed paths: average_stress (src/flowfield/stress.rs:60-96),
// DirectorField::from_distribution (src/polarization/director.rs:36-61) and
// the density of src/bin/simulation/mod.rs:312-316.
//
// A block takes kCTile consecutive cells, one thread per cell.  Their counts
// are contiguous in HBM ([cell][phi][theta]); the block stages them, 32
// angles of every cell at a time, into shared memory with coalesced loads
// (16 bytes wide where the rows allow it), each row padded to an odd stride
// so that thread t reading angle a of its own cell hits bank
// (t * stride + a) mod 32 -- 32 different banks.  The small tiles (64 cells,
// 32 angles: 8 KB of counts) let many blocks share an SM, so that one
// block's loads overlap another's arithmetic.  Thread t then runs over its
// cell's angles in order while the angle kernels of the chunk are broadcast
// from shared memory (every thread reads the same angle at the same time).
// The histogram is read once, coalesced.
//
// FP64 path.  GB300 executes FP64 at 1/64 of the FP32 rate, so the products
// K_j(a) * f(count) are not formed in FP64.  At set-up every kernel component
// is split into four signed 12-bit integer slices relative to its largest
// magnitude (kernel_slices, host side):
//     K_j(a) = 2^(E_j - 48) * (m_j1(a) 2^36 + m_j2(a) 2^24 + m_j3(a) 2^12 + m_j4(a))
// up to 2^-49 max_a |K_j(a)|.  While a cell holds at most 2^12 particles,
// every product m * count and every partial sum over the cell's angles is an
// integer of magnitude at most 2^24, exact in FP32.  The four slice sums
// combine exactly in a 64-bit integer; one conversion and one multiplication
// by 2^(E_j - 48) * measure * V / D give the component in FP64.  A cell with
// more particles runs the FP64 loop instead.  The result differs from the
// reference's sum of K_j(a) * ((count / D) * V) by a few ulps.
//
// FP32 path.  Products K_j(a) * count in FP32, scaled once by
// measure * V / D (or by the denoised distribution's scale).  The
// per-component sums that the mean handling needs are formed in a fixed
// order -- float-pair warp sums, block sums in FP64 in warp order, and the
// last block to finish adds the blocks' sums in block order -- so they are
// the same bit for bit from run to run.
#include "kernels.cuh"
#include "mixed.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>

#include <cmath>

namespace ss {

namespace {

constexpr int kCTile = 64;     // cells (= threads) per block
constexpr int kAngChunk = 32;  // angles of every cell staged at a time
constexpr int kSliceW = 48;     // floats per angle of the FP64 path's slice table: 12 components x 4 slices
constexpr uint32_t kExactCells = 4096;  // particles per cell below which the FP32 slice sums are exact

struct Staging {
    int na;      // angles per cell
    int stride;  // padded row stride of the staged counts (odd)
    int vec;     // rows are read 16 bytes wide: na a multiple of 4 (so every staged segment is 16-byte aligned)
};

// counts (or FP32 distribution bits) of rows r < tc, angles a0 .. a0 + ach,
// from src = base of row 0, into tile[r * stride + a - a0].  With 16-byte
// loads a row segment of 32 angles is 8 quads: quad q of the tile lands at
// row q / 8, word 4 (q % 8), and with the stride of 33 words a warp's 32
// quads (4 rows x 8) store to 32 different banks.
__device__ __forceinline__ void stage_rows(const uint32_t *__restrict__ src, const Staging &S, int a0, int ach,
                                           int tc, uint32_t *__restrict__ tile) {
    const int tid = threadIdx.x;
    if (S.vec && (ach & 3) == 0) {
        const int qpr = ach >> 2, nq = tc * qpr, rq = S.na >> 2;
        const uint4 *s4 = reinterpret_cast<const uint4 *>(src + a0);
#pragma unroll 4
        for (int q = tid; q < nq; q += kCTile) {
            const int r = q / qpr, cq = q - r * qpr;
            const uint4 v = __ldg(s4 + (long long)r * rq + cq);
            uint32_t *d = tile + r * S.stride + 4 * cq;
            d[0] = v.x;
            d[1] = v.y;
            d[2] = v.z;
            d[3] = v.w;
        }
    } else {
        const int nw = tc * ach;
        for (int i = tid; i < nw; i += kCTile) {
            const int r = i / ach, a = i - r * ach;
            tile[r * S.stride + a] = __ldg(src + (long long)r * S.na + a0 + a);
        }
    }
}

// Float pairs (hi, lo), an unevaluated sum of two floats (about 48 bits),
// added by error-free transformations (Knuth's two-sum, then a fast two-sum
// to renormalise); every operation is on the FP32 pipe.
struct FPair {
    float hi, lo;
};
__device__ __forceinline__ FPair pair_add(FPair a, FPair b) {
    const float s = a.hi + b.hi, bb = s - a.hi;
    const float e = (a.hi - (s - bb)) + (b.hi - bb);  // (a.hi + b.hi) - s exactly
    const float lo = (a.lo + b.lo) + e;
    const float h = s + lo;
    return FPair{h, lo - (h - s)};
}
// the pair summed over the warp in a fixed butterfly order (every lane ends
// with the same pair)
__device__ __forceinline__ FPair warp_pair_sum(FPair v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const FPair w{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
        v = pair_add(v, w);
    }
    return v;
}

// ---------------------------------------------------------------------------
// FP64 path
// ---------------------------------------------------------------------------
template <bool STRESS, bool MAG>
__global__ void __launch_bounds__(kCTile) k_contract_x(const uint32_t *__restrict__ counts,
                                                       const float *__restrict__ kslice,
                                                       const double *__restrict__ factor,
                                                       const double *__restrict__ kern,
                                                       const double *__restrict__ lut, int lut_n, DevParams P,
                                                       Staging S, double *__restrict__ fwd,
                                                       double *__restrict__ table, int tstride,
                                                       uint32_t *__restrict__ cellcount, double dfac) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int na = S.na;
    float *ks = reinterpret_cast<float *>(smem);  // [chunk angle][48]
    uint32_t *tile = reinterpret_cast<uint32_t *>(ks + (na < kAngChunk ? na : kAngChunk) * kSliceW);
    const int tid = threadIdx.x, cell0 = blockIdx.x * kCTile;
    const int tc = min(kCTile, P.ncell - cell0);
    const bool live = tid < tc;
    const int cell = cell0 + tid;
    float acc[48];
#pragma unroll
    for (int j = 0; j < 48; ++j) acc[j] = 0.f;
    uint32_t csum = 0;
    const uint32_t *src = counts + (long long)cell0 * na;
    for (int a0 = 0; a0 < na; a0 += kAngChunk) {
        const int ach = min(kAngChunk, na - a0);
        __syncthreads();  // the previous chunk is consumed
        {
            const float4 *g = reinterpret_cast<const float4 *>(kslice + (long long)a0 * kSliceW);
            float4 *d = reinterpret_cast<float4 *>(ks);
            for (int i = tid; i < ach * (kSliceW / 4); i += kCTile) d[i] = __ldg(g + i);
        }
        stage_rows(src, S, a0, ach, tc, tile);
        __syncthreads();
        if (live) {
            const uint32_t *row = tile + tid * S.stride;
            for (int a = 0; a < ach; ++a) {
                const uint32_t n = row[a];
                csum += n;
                // the exact float of n < 2^23 from its bits; larger counts exceed
                // the exactness bound and are redone in FP64 below
                const float c = __uint_as_float((n & 0x7FFFFFu) | 0x4B000000u) - 8388608.f;
                const float4 *k4 = reinterpret_cast<const float4 *>(ks + a * kSliceW);
                if (STRESS) {
#pragma unroll
                    for (int q = 0; q < 9; ++q) {
                        const float4 k = k4[q];
                        acc[4 * q + 0] = fmaf(k.x, c, acc[4 * q + 0]);
                        acc[4 * q + 1] = fmaf(k.y, c, acc[4 * q + 1]);
                        acc[4 * q + 2] = fmaf(k.z, c, acc[4 * q + 2]);
                        acc[4 * q + 3] = fmaf(k.w, c, acc[4 * q + 3]);
                    }
                }
                if (MAG) {
#pragma unroll
                    for (int q = 9; q < 12; ++q) {
                        const float4 k = k4[q];
                        acc[4 * q + 0] = fmaf(k.x, c, acc[4 * q + 0]);
                        acc[4 * q + 1] = fmaf(k.y, c, acc[4 * q + 1]);
                        acc[4 * q + 2] = fmaf(k.z, c, acc[4 * q + 2]);
                        acc[4 * q + 3] = fmaf(k.w, c, acc[4 * q + 3]);
                    }
                }
            }
        }
    }
    if (!live) return;
    double sig[12];
    if (csum <= kExactCells) {
#pragma unroll
        for (int j = 0; j < 12; ++j) {
            if ((j < 9 && STRESS) || (j >= 9 && MAG)) {
                const long long A = (long long)__float2int_rn(acc[4 * j + 0]) * (1ll << 36) +
                                    (long long)__float2int_rn(acc[4 * j + 1]) * (1ll << 24) +
                                    (long long)__float2int_rn(acc[4 * j + 2]) * (1ll << 12) +
                                    (long long)__float2int_rn(acc[4 * j + 3]);
                sig[j] = (double)A * factor[j];
            }
        }
    } else {
        // a crowded cell: the reference's FP64 sum of K_j(a) * ((count / D) * V), times measure
        double s[12];
#pragma unroll
        for (int j = 0; j < 12; ++j) s[j] = 0.0;
        const long long row = (long long)cell * na;
        for (int a = 0; a < na; ++a) {
            const uint32_t n = counts[row + a];
            const double f = ((int)n < lut_n && (int)n >= 0) ? __ldg(lut + n) : ((double)n / P.dist_den) * P.volume;
            if (STRESS) {
#pragma unroll
                for (int j = 0; j < 9; ++j) s[j] = fma(kern[j * na + a], f, s[j]);
            }
            if (MAG) {
#pragma unroll
                for (int j = 9; j < 12; ++j) s[j] = fma(kern[j * na + a], f, s[j]);
            }
        }
#pragma unroll
        for (int j = 0; j < 12; ++j) sig[j] = s[j] * P.measure;
    }
    if (STRESS) {
#pragma unroll
        for (int j = 0; j < 9; ++j) fwd[(long long)j * P.cstride + cell] = sig[j];
    }
    if (MAG) {
#pragma unroll
        for (int j = 9; j < 12; ++j) fwd[(long long)j * P.cstride + cell] = sig[j];
    }
    // (count / D) V dtheta dphi with the factor V / D dtheta dphi formed once: a
    // division per cell costs ~20 FP64 operations on GB300's narrow FP64 pipe
    const double dens = (double)csum * dfac;
    table[(long long)cell * tstride + T_DIFF] = sqrt(2.0 * P.dt * (P.Dt + P.volex * dens));
    if (tstride == TABLE_STRIDE_MAG) table[(long long)cell * tstride + T_DENS] = dens;
    cellcount[cell] = csum;
}

// ---------------------------------------------------------------------------
// FP32 mixed path.  DIST: the tile holds the bits of an FP32 distribution
// (the denoised histogram) instead of counts.  A persistent grid (a few
// blocks per SM) walks the cell tiles in a fixed pattern; every thread keeps
// float-pair sums of its cells' components, the block adds its threads'
// pairs in a fixed order, and the last block to finish adds the blocks'
// pairs in block order and writes the FP64 sums.  No FP64 arithmetic runs
// per cell (GB300 executes FP64 at 1/64 of the FP32 rate).
// ---------------------------------------------------------------------------
template <bool STRESS, bool MAG, bool DIST>
__global__ void __launch_bounds__(kCTile) k_contract_f(const uint32_t *__restrict__ src_bins,
                                                       const float *__restrict__ kern, MixedParams M, Staging S,
                                                       float scale, float dscale, float *__restrict__ fwd,
                                                       float *__restrict__ table, int tstride,
                                                       float2 *__restrict__ partials, unsigned *__restrict__ done,
                                                       double *__restrict__ sums) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ FPair red[kCTile / 32][12];
    __shared__ bool s_last;
    const int na = S.na;
    float *kf = reinterpret_cast<float *>(smem);  // [chunk angle][12]
    uint32_t *tile = reinterpret_cast<uint32_t *>(kf + (na < kAngChunk ? na : kAngChunk) * 12);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nc = M.ncell, ntiles = (nc + kCTile - 1) / kCTile;
    FPair tot[12];
#pragma unroll
    for (int j = 0; j < 12; ++j) tot[j] = FPair{0.f, 0.f};
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int cell0 = t * kCTile, tc = min(kCTile, nc - cell0);
        const bool live = tid < tc;
        const int cell = cell0 + tid;
        float acc[12];
#pragma unroll
        for (int j = 0; j < 12; ++j) acc[j] = 0.f;
        float dsum = 0.f;
        uint32_t csum = 0;
        const uint32_t *src = src_bins + (long long)cell0 * na;
        for (int a0 = 0; a0 < na; a0 += kAngChunk) {
            const int ach = min(kAngChunk, na - a0);
            __syncthreads();
            // the chunk's angle kernels, transposed to [angle][component]
            for (int i = tid; i < 12 * ach; i += kCTile) {
                const int j = i / ach, a = i - j * ach;
                kf[a * 12 + j] = __ldg(kern + (long long)j * na + a0 + a);
            }
            stage_rows(src, S, a0, ach, tc, tile);
            __syncthreads();
            if (live) {
                const uint32_t *row = tile + tid * S.stride;
                for (int a = 0; a < ach; ++a) {
                    const uint32_t w = row[a];
                    float f;
                    if (DIST) {
                        f = __uint_as_float(w);
                        dsum += f;
                    } else {
                        f = __uint2float_rn(w);
                        csum += w;
                    }
                    const float4 *k4 = reinterpret_cast<const float4 *>(kf + a * 12);
                    if (STRESS) {
#pragma unroll
                        for (int q = 0; q < 2; ++q) {
                            const float4 k = k4[q];
                            acc[4 * q + 0] = fmaf(k.x, f, acc[4 * q + 0]);
                            acc[4 * q + 1] = fmaf(k.y, f, acc[4 * q + 1]);
                            acc[4 * q + 2] = fmaf(k.z, f, acc[4 * q + 2]);
                            acc[4 * q + 3] = fmaf(k.w, f, acc[4 * q + 3]);
                        }
                    }
                    if (STRESS || MAG) {
                        const float4 k = k4[2];
                        if (STRESS) acc[8] = fmaf(k.x, f, acc[8]);
                        if (MAG) {
                            acc[9] = fmaf(k.y, f, acc[9]);
                            acc[10] = fmaf(k.z, f, acc[10]);
                            acc[11] = fmaf(k.w, f, acc[11]);
                        }
                    }
                }
            }
        }
        if (live) {
            float out[12];
#pragma unroll
            for (int j = 0; j < 12; ++j) out[j] = acc[j] * scale;
            if (STRESS) {
#pragma unroll
                for (int j = 0; j < 9; ++j) fwd[(long long)j * M.cstride + cell] = out[j];
            }
            if (MAG) {
#pragma unroll
                for (int j = 9; j < 12; ++j) fwd[(long long)j * M.cstride + cell] = out[j];
            }
#pragma unroll
            for (int j = 0; j < 12; ++j)
                if ((j < 9 && STRESS) || (j >= 9 && MAG)) tot[j] = pair_add(tot[j], FPair{out[j], 0.f});
            // density = (count / D) V dtheta dphi; dscale = V / D dtheta dphi (or the distribution's scale)
            const float dens = DIST ? dsum * dscale : (float)csum * dscale;
            table[(long long)cell * tstride + T_DIFF] = sqrtf(M.two_dt * (M.Dt + M.volex * dens));
        }
    }
    // the block's pairs: warp butterflies, then the warps in order
#pragma unroll
    for (int j = 0; j < 12; ++j) {
        if ((j < 9 && STRESS) || (j >= 9 && MAG)) {
            const FPair v = warp_pair_sum(tot[j]);
            if (lane == 0) red[warp][j] = v;
        }
    }
    __syncthreads();
    if (tid < 12 && ((tid < 9 && STRESS) || (tid >= 9 && MAG))) {
        FPair v = red[0][tid];
#pragma unroll
        for (int w = 1; w < kCTile / 32; ++w) v = pair_add(v, red[w][tid]);
        partials[(long long)blockIdx.x * 12 + tid] = make_float2(v.hi, v.lo);
        __threadfence();
    }
    __syncthreads();
    if (tid == 0) s_last = atomicAdd(done, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!s_last) return;
    // the last block: each thread adds a fixed, strided subset of the blocks'
    // pairs, then the threads' pairs in a fixed tree
    __threadfence();
    for (int j = 0; j < 12; ++j) {
        if (!((j < 9 && STRESS) || (j >= 9 && MAG))) continue;
        FPair v{0.f, 0.f};
        for (int b = tid; b < (int)gridDim.x; b += kCTile) {
            const float2 q = __ldcg(partials + (long long)b * 12 + j);
            v = pair_add(v, FPair{q.x, q.y});
        }
        v = warp_pair_sum(v);
        __syncthreads();
        if (lane == 0) red[warp][0] = v;
        __syncthreads();
        if (tid == 0) {
            FPair t = red[0][0];
#pragma unroll
            for (int w = 1; w < kCTile / 32; ++w) t = pair_add(t, red[w][0]);
            sums[j] = (double)t.hi + (double)t.lo;
        }
    }
    if (tid == 0) *done = 0u;  // ready for the next launch
}

// ---------------------------------------------------------------------------
// FP32 mixed path, TMA-staged (rows of a multiple of 16 bytes).  The
// histogram, viewed as a 2-D tensor [ncell][nang] of u32, is copied tile by
// tile -- 128 cells x 32 angles, 16 KB -- by the tensor memory accelerator
// (cp.async.bulk.tensor.2d) into one of two shared-memory buffers, each
// completing on its own mbarrier, two tiles ahead of the arithmetic: one
// elected thread issues the copies, no thread spends instructions on
// addresses, and the copies overlap the FMAs.  Angles past the row end and
// cells past the grid arrive as zeros (the copy's out-of-bounds fill),
// against zero-padded angle kernels.  The buffers keep the tensor's dense
// layout (rows of 32 words); thread t takes rows t and t + 64 and visits
// their angles from a = t mod 32 on, so a warp's 32 reads hit 32 banks, and
// the angle kernels ([angle][12] floats, staged once per block) are then read
// 48 bytes apart, which also maps a warp's 16-byte reads to distinct banks;
// each such read serves both of the thread's cells, halving the shared-memory
// traffic that bounds the kernel.  Every mbarrier
// wait is bounded: on a timeout the kernel sets bit kErrTmaTimeout of err,
// waits (bounded) for its own copies and leaves the sums wrong but the
// launch protocol intact.
// ---------------------------------------------------------------------------
constexpr int kTmaCells = 2 * kCTile;                // cells per tile: two per thread
constexpr int kTmaBytes = kTmaCells * kAngChunk * 4;  // one tile: 16 KB
constexpr int kTmaBlocksPerSM = 4;                    // 2 x 16 KB + the angle kernels per block
constexpr uint32_t kWaitPolls = 1u << 22;
constexpr unsigned kErrTmaTimeout = 0x100u;

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint32_t a, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(a), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t a, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(a), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t a, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t a, uint32_t parity) {
    for (uint32_t i = 0; i < kWaitPolls; ++i)
        if (mbar_try_wait(a, parity)) return true;
    return false;
}
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t mbar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];\n" ::"r"(
            dst),
        "l"(map), "r"(x), "r"(y), "r"(mbar)
        : "memory");
}

template <bool STRESS, bool MAG, bool DIST>
__global__ void __launch_bounds__(kCTile) k_contract_t(const __grid_constant__ CUtensorMap tmap,
                                                       const float *__restrict__ kern_t, int na_pad, MixedParams M,
                                                       float scale, float dscale, float *__restrict__ fwd,
                                                       float *__restrict__ table, int tstride,
                                                       float2 *__restrict__ partials, unsigned *__restrict__ done,
                                                       double *__restrict__ sums, unsigned *__restrict__ err) {
    extern __shared__ __align__(1024) unsigned char smem_tma[];  // TMA destinations: 128-byte aligned at least
    uint32_t *buf = reinterpret_cast<uint32_t *>(smem_tma);           // 2 tiles of [64][32] words
    float *kf = reinterpret_cast<float *>(smem_tma + 2 * kTmaBytes);  // [na_pad][12]
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ FPair red[kCTile / 32][12];
    __shared__ bool s_last;
    __shared__ int s_fail;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nc = M.ncell, ntiles = (nc + kTmaCells - 1) / kTmaCells, nch = na_pad / kAngChunk;
    const int my_tiles = (int)blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    const int nitems = my_tiles * nch;
    for (int i = tid; i < na_pad * 3; i += kCTile)
        reinterpret_cast<float4 *>(kf)[i] = __ldg(reinterpret_cast<const float4 *>(kern_t) + i);
    const uint32_t mb0 = smem_addr(&mbar[0]), buf0 = smem_addr(buf);
    if (tid == 0) {
        mbar_init(mb0, 1);
        mbar_init(mb0 + 8, 1);
        s_fail = 0;
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    auto issue = [&](int k) {
        const int m = k / nch, c = k - m * nch, t = (int)blockIdx.x + m * (int)gridDim.x;
        const uint32_t b = (uint32_t)(k & 1);
        mbar_expect_tx(mb0 + 8 * b, (uint32_t)kTmaBytes);
        tma_load_2d(buf0 + b * (uint32_t)kTmaBytes, &tmap, c * kAngChunk, t * kTmaCells, mb0 + 8 * b);
    };
    if (tid == 0) {
        if (nitems > 0) issue(0);
        if (nitems > 1) issue(1);
    }
    FPair tot[12];
#pragma unroll
    for (int j = 0; j < 12; ++j) tot[j] = FPair{0.f, 0.f};
    float acc[2][12];
    float dsum[2];
    uint32_t csum[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
#pragma unroll
        for (int j = 0; j < 12; ++j) acc[h][j] = 0.f;
        dsum[h] = 0.f;
        csum[h] = 0;
    }
    int k = 0;
    for (; k < nitems; ++k) {
        const int m = k / nch, c = k - m * nch;
        if (c == 0) {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
#pragma unroll
                for (int j = 0; j < 12; ++j) acc[h][j] = 0.f;
                dsum[h] = 0.f;
                csum[h] = 0;
            }
        }
        // every thread observes the copy's completion (which makes its bytes visible to it)
        if (!mbar_wait_bounded(mb0 + 8 * (uint32_t)(k & 1), (uint32_t)((k >> 1) & 1))) s_fail = 1;
        __syncthreads();
        if (s_fail) break;
        const uint32_t *row0 = buf + (k & 1) * (kTmaBytes / 4) + tid * kAngChunk;
        const uint32_t *row1 = row0 + kCTile * kAngChunk;
        const float *kc = kf + c * kAngChunk * 12;
#pragma unroll 2
        for (int i = 0; i < kAngChunk; ++i) {
            const int a = (i + tid) & (kAngChunk - 1);
            const uint32_t w0 = row0[a], w1 = row1[a];
            float f0, f1;
            if (DIST) {
                f0 = __uint_as_float(w0);
                f1 = __uint_as_float(w1);
                dsum[0] += f0;
                dsum[1] += f1;
            } else {
                f0 = __uint2float_rn(w0);
                f1 = __uint2float_rn(w1);
                csum[0] += w0;
                csum[1] += w1;
            }
            const float4 *k4 = reinterpret_cast<const float4 *>(kc + a * 12);
            if (STRESS) {
#pragma unroll
                for (int q = 0; q < 2; ++q) {
                    const float4 kv = k4[q];
                    acc[0][4 * q + 0] = fmaf(kv.x, f0, acc[0][4 * q + 0]);
                    acc[0][4 * q + 1] = fmaf(kv.y, f0, acc[0][4 * q + 1]);
                    acc[0][4 * q + 2] = fmaf(kv.z, f0, acc[0][4 * q + 2]);
                    acc[0][4 * q + 3] = fmaf(kv.w, f0, acc[0][4 * q + 3]);
                    acc[1][4 * q + 0] = fmaf(kv.x, f1, acc[1][4 * q + 0]);
                    acc[1][4 * q + 1] = fmaf(kv.y, f1, acc[1][4 * q + 1]);
                    acc[1][4 * q + 2] = fmaf(kv.z, f1, acc[1][4 * q + 2]);
                    acc[1][4 * q + 3] = fmaf(kv.w, f1, acc[1][4 * q + 3]);
                }
            }
            if (STRESS || MAG) {
                const float4 kv = k4[2];
                if (STRESS) {
                    acc[0][8] = fmaf(kv.x, f0, acc[0][8]);
                    acc[1][8] = fmaf(kv.x, f1, acc[1][8]);
                }
                if (MAG) {
                    acc[0][9] = fmaf(kv.y, f0, acc[0][9]);
                    acc[0][10] = fmaf(kv.z, f0, acc[0][10]);
                    acc[0][11] = fmaf(kv.w, f0, acc[0][11]);
                    acc[1][9] = fmaf(kv.y, f1, acc[1][9]);
                    acc[1][10] = fmaf(kv.z, f1, acc[1][10]);
                    acc[1][11] = fmaf(kv.w, f1, acc[1][11]);
                }
            }
        }
        __syncthreads();  // the buffer is consumed: the copy two tiles ahead may overwrite it
        if (tid == 0 && k + 2 < nitems) {
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            issue(k + 2);
        }
        if (c == nch - 1) {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int cell = ((int)blockIdx.x + m * (int)gridDim.x) * kTmaCells + h * kCTile + tid;
                if (cell < nc) {
                    float out[12];
#pragma unroll
                    for (int j = 0; j < 12; ++j) out[j] = acc[h][j] * scale;
                    if (STRESS) {
#pragma unroll
                        for (int j = 0; j < 9; ++j) fwd[(long long)j * M.cstride + cell] = out[j];
                    }
                    if (MAG) {
#pragma unroll
                        for (int j = 9; j < 12; ++j) fwd[(long long)j * M.cstride + cell] = out[j];
                    }
#pragma unroll
                    for (int j = 0; j < 12; ++j)
                        if ((j < 9 && STRESS) || (j >= 9 && MAG)) tot[j] = pair_add(tot[j], FPair{out[j], 0.f});
                    const float dens = DIST ? dsum[h] * dscale : (float)csum[h] * dscale;
                    table[(long long)cell * tstride + T_DIFF] = sqrtf(M.two_dt * (M.Dt + M.volex * dens));
                }
            }
        }
    }
    if (s_fail) {
        // the copies this block issued and did not see land: wait for them (bounded) before leaving
        if (tid == 0) {
            atomicOr(err, kErrTmaTimeout);
            for (int q = k; q < nitems && q < k + 2; ++q)
                mbar_wait_bounded(mb0 + 8 * (uint32_t)(q & 1), (uint32_t)((q >> 1) & 1));
        }
        __syncthreads();
    }
    // the block's pairs: warp butterflies, then the warps in order
#pragma unroll
    for (int j = 0; j < 12; ++j) {
        if ((j < 9 && STRESS) || (j >= 9 && MAG)) {
            const FPair v = warp_pair_sum(tot[j]);
            if (lane == 0) red[warp][j] = v;
        }
    }
    __syncthreads();
    if (tid < 12 && ((tid < 9 && STRESS) || (tid >= 9 && MAG))) {
        FPair v = red[0][tid];
#pragma unroll
        for (int w = 1; w < kCTile / 32; ++w) v = pair_add(v, red[w][tid]);
        partials[(long long)blockIdx.x * 12 + tid] = make_float2(v.hi, v.lo);
        __threadfence();
    }
    __syncthreads();
    if (tid == 0) s_last = atomicAdd(done, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    for (int j = 0; j < 12; ++j) {
        if (!((j < 9 && STRESS) || (j >= 9 && MAG))) continue;
        FPair v{0.f, 0.f};
        for (int b = tid; b < (int)gridDim.x; b += kCTile) {
            const float2 q = __ldcg(partials + (long long)b * 12 + j);
            v = pair_add(v, FPair{q.x, q.y});
        }
        v = warp_pair_sum(v);
        __syncthreads();
        if (lane == 0) red[warp][0] = v;
        __syncthreads();
        if (tid == 0) {
            FPair t = red[0][0];
#pragma unroll
            for (int w = 1; w < kCTile / 32; ++w) t = pair_add(t, red[w][0]);
            sums[j] = (double)t.hi + (double)t.lo;
        }
    }
    if (tid == 0) *done = 0u;
}

Staging make_staging(int na) {
    Staging S;
    S.na = na;
    const int ach = na < kAngChunk ? na : kAngChunk;
    S.stride = ach | 1;
    S.vec = (na & 3) == 0;
    return S;
}

size_t smem_x(int na) {
    const int ach = na < kAngChunk ? na : kAngChunk;
    return (size_t)ach * kSliceW * sizeof(float) + (size_t)kCTile * (ach | 1) * sizeof(uint32_t);
}
size_t smem_f(int na) {
    const int ach = na < kAngChunk ? na : kAngChunk;
    return (size_t)ach * 12 * sizeof(float) + (size_t)kCTile * (ach | 1) * sizeof(uint32_t);
}

unsigned tiles(int ncell) { return (unsigned)((ncell + kCTile - 1) / kCTile); }

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
void kernel_slices(const std::vector<double> &K, int na, double measure_v_over_d, std::vector<float> &slices,
                   std::vector<double> &factor) {
    slices.assign((size_t)na * kSliceW, 0.f);
    factor.assign(12, 0.0);
    for (int j = 0; j < 12; ++j) {
        double mx = 0.0;
        for (int a = 0; a < na; ++a) mx = std::fmax(mx, std::fabs(K[(size_t)j * na + a]));
        if (!(mx > 0.0) || !std::isfinite(mx)) continue;  // an all-zero component stays zero
        const int E = std::ilogb(mx) + 1;                 // max |K_j| < 2^E
        for (int a = 0; a < na; ++a) {
            // v = K 2^(12 - E), |v| < 2^12; four roundings to integers, each
            // remainder (exact) scaled by 2^12 for the next slice
            double v = std::ldexp(K[(size_t)j * na + a], 12 - E);
            for (int s = 0; s < 4; ++s) {
                const double m = std::nearbyint(v);
                slices[(size_t)a * kSliceW + 4 * j + s] = (float)m;
                v = std::ldexp(v - m, 12);
            }
        }
        factor[j] = std::ldexp(1.0, E - 48) * measure_v_over_d;
    }
}

cudaError_t contract_prepare() {
    // the largest dynamic shared memory any grid needs (angle chunks of kAngChunk)
    const int bx = (int)smem_x(kAngChunk), bf = (int)smem_f(kAngChunk);
    cudaError_t e = cudaSuccess;
    auto set = [&](const void *f, int bytes) {
        if (e == cudaSuccess) e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    };
    set((const void *)k_contract_x<true, true>, bx);
    set((const void *)k_contract_x<true, false>, bx);
    set((const void *)k_contract_x<false, true>, bx);
    set((const void *)k_contract_f<true, true, false>, bf);
    set((const void *)k_contract_f<true, false, false>, bf);
    set((const void *)k_contract_f<false, true, false>, bf);
    set((const void *)k_contract_f<true, true, true>, bf);
    set((const void *)k_contract_f<true, false, true>, bf);
    set((const void *)k_contract_f<false, true, true>, bf);
    const int bt = 80 * 1024;
    set((const void *)k_contract_t<true, true, false>, bt);
    set((const void *)k_contract_t<true, false, false>, bt);
    set((const void *)k_contract_t<false, true, false>, bt);
    set((const void *)k_contract_t<true, true, true>, bt);
    set((const void *)k_contract_t<true, false, true>, bt);
    set((const void *)k_contract_t<false, true, true>, bt);
    return e;
}

void launch_contract_x(cudaStream_t s, bool stress, bool mag, const uint32_t *counts, const float *kslice,
                       const double *factor, const double *kern, const double *lut, int lut_n, const DevParams &P,
                       double *fwd, double *table, int tstride, uint32_t *cellcount) {
    const Staging S = make_staging(P.nang);
    const size_t sm = smem_x(P.nang);
    const unsigned b = tiles(P.ncell);
    const double dfac = (P.volume / P.dist_den) * P.dthph;
#define SS_CX(ST, MG)                                                                                        \
    k_contract_x<ST, MG><<<b, kCTile, sm, s>>>(counts, kslice, factor, kern, lut, lut_n, P, S, fwd, table, \
                                               tstride, cellcount, dfac)
    if (stress && mag) SS_CX(true, true);
    else if (stress) SS_CX(true, false);
    else SS_CX(false, true);
#undef SS_CX
}

// the persistent grid of the FP32 contraction: at most kMBlocksPerSM blocks per SM
constexpr int kMBlocksPerSM = 8;
unsigned contract_m_blocks(int ncell, int sms) {
    const unsigned t = tiles(ncell), cap = (unsigned)(kMBlocksPerSM * (sms > 0 ? sms : 1));
    return t < cap ? t : cap;
}

// the angle kernels [12][na] transposed to [angle][12], zero rows up to a
// multiple of 32 angles (the TMA-staged contraction)
void kernel_transposed(const std::vector<double> &K, int na, std::vector<float> &out) {
    const int pad = (na + kAngChunk - 1) / kAngChunk * kAngChunk;
    out.assign((size_t)pad * 12, 0.f);
    for (int a = 0; a < na; ++a)
        for (int j = 0; j < 12; ++j) out[(size_t)a * 12 + j] = (float)K[(size_t)j * na + a];
}

// the tensor map of a histogram (or an FP32 distribution) [ncell][na] of
// 4-byte elements, tiles of 64 cells x 32 angles; false when the rows are not
// a multiple of 16 bytes (na % 4 != 0), the base is not 16-byte aligned, or
// the driver's encoder is unavailable
bool make_bins_tmap(CUtensorMap *map, const void *base, int ncell, int na) {
    // tiles of kTmaCells cells x kAngChunk angles
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (!encode) {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !fn)
            return false;
        encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }
    if (na % 4 != 0 || na > (1 << 20) || ncell < 1 || ((uintptr_t)base & 15u)) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)na, (cuuint64_t)ncell};
    const cuuint64_t strides[1] = {(cuuint64_t)na * 4u};
    const cuuint32_t box[2] = {(cuuint32_t)kAngChunk, (cuuint32_t)kTmaCells};
    const cuuint32_t estr[2] = {1u, 1u};
    const CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, const_cast<void *>(base), dims, strides, box,
                              estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

static size_t smem_t(int na_pad) { return 2u * kTmaBytes + (size_t)na_pad * 12 * sizeof(float); }
bool contract_tma_fits(int na) {
    const int pad = (na + kAngChunk - 1) / kAngChunk * kAngChunk;
    return smem_t(pad) <= 80 * 1024;
}

void launch_contract_m(cudaStream_t s, bool stress, bool mag, const uint32_t *counts, const float *kern,
                       const MixedParams &M, float *fwd, float *table, int tstride, float2 *partials,
                       unsigned *done, double *sums, int sms, const float *dist, float fscale,
                       const CUtensorMap *tmap, const float *kern_t, unsigned *err) {
    const unsigned b = contract_m_blocks(M.ncell, sms);
    const bool fd = dist != nullptr;
    const uint32_t *src = fd ? reinterpret_cast<const uint32_t *>(dist) : counts;
    // counts: f = count, scaled by measure * V / D; a distribution: f = value, scaled by measure * fscale
    const float scale = fd ? M.measure * fscale : (float)((double)M.measure * (M.volume / M.dist_den));
    const float dscale = fd ? fscale * M.dthph : (float)((M.volume / M.dist_den) * (double)M.dthph);
    if (tmap && kern_t && err) {
        const int pad = (M.nang + kAngChunk - 1) / kAngChunk * kAngChunk;
        const size_t sm = smem_t(pad);
        const unsigned tt = (unsigned)((M.ncell + kTmaCells - 1) / kTmaCells);
        const unsigned cap = (unsigned)(kTmaBlocksPerSM * (sms > 0 ? sms : 1));
        const unsigned b = tt < cap ? tt : cap;  // every block resident: tiles are split evenly
#define SS_CT(ST, MG, D)                                                                                       \
    k_contract_t<ST, MG, D><<<b, kCTile, sm, s>>>(*tmap, kern_t, pad, M, scale, dscale, fwd, table, tstride, \
                                                  partials, done, sums, err)
        if (stress && mag) { if (fd) SS_CT(true, true, true); else SS_CT(true, true, false); }
        else if (stress) { if (fd) SS_CT(true, false, true); else SS_CT(true, false, false); }
        else { if (fd) SS_CT(false, true, true); else SS_CT(false, true, false); }
#undef SS_CT
        return;
    }
    const Staging S = make_staging(M.nang);
    const size_t sm = smem_f(M.nang);
#define SS_CF(ST, MG, D)                                                                                    \
    k_contract_f<ST, MG, D><<<b, kCTile, sm, s>>>(src, kern, M, S, scale, dscale, fwd, table, tstride,   \
                                                  partials, done, sums)
    if (stress && mag) { if (fd) SS_CF(true, true, true); else SS_CF(true, true, false); }
    else if (stress) { if (fd) SS_CF(true, false, true); else SS_CF(true, false, false); }
    else { if (fd) SS_CF(false, true, true); else SS_CF(false, true, false); }
#undef SS_CF
}

}  // namespace ss
