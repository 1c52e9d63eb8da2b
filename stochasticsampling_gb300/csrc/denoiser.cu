// denoiser.cu -- the learned histogram denoiser: a 3-D CNN (4 convolutions
// of 3x3x3 with periodic padding, 32 channels, ReLU, residual) that maps a
// low-particle-count histogram on the (x, y, phi) grid to an estimate of the
// high-count distribution before the stress / Stokes solve.
//
// Activations are BF16, channels last, in the layout [x][phi][y][32], so
// that a line along y (the 128 voxels of one tile) is contiguous.  The
// 32 -> 32 convolutions are implicit GEMMs on the 5th-generation tensor
// cores: per tile (x, phi, 128 consecutive y), D[128 x 32] = sum over the 27
// taps of A_tap[128 x 32] W_tap[32 x 32]^T, BF16 operands in shared memory,
// FP32 accumulator in tensor memory, one elected thread issuing tcgen05.mma
// (M = 128, N = 32, K = 16).  A CTA walks along phi: it keeps the lines
// (x + dx, phi + dphi) of the current tile in a ring of 12 line buffers (3
// x-planes x 4 positions along phi), each line with one halo row at either
// end (130 rows), and loads only the 3 lines the next tile adds; the 27 taps
// are descriptor offsets into those lines (the y shift is a 16-byte row
// offset), so every activation row is read from global memory about 3 times
// instead of 27.  Lines are copied with cp.async; a tile's 54 MMAs are issued
// back to back and committed to an mbarrier.  The epilogue reads the
// accumulator with tcgen05.ld (one voxel's 32 channels per thread), adds the
// bias and applies ReLU (or the ReLU derivative of a reference tensor, for
// the backward pass).
//
// Shared-memory operand layouts (K-major, no swizzle).  A line: for each of
// its 4 K chunks (8 channels, 16 bytes) the 130 rows at a 16-byte stride, so
// row groups are 128 B apart (stride offset) and K chunks 2080 B (leading
// offset).  Weights: per tap 32 rows x 4 chunks in 8 x 16 B core matrices,
// leading offset 128 B, stride offset 512 B.  Every wait is bounded: on a
// timeout the kernel records an error, waits for its own copies, frees its
// tensor memory and returns.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <random>
#include <string>
#include <vector>

#include "../../include/ssgpu.h"
#include "common.cuh"

namespace ss {
void record_error(const char *msg);
}

namespace {

constexpr int kC = 32;                       // channels
constexpr int kTaps = 27;                    // 3 x 3 x 3
constexpr int kTileM = 128;                  // voxels per tile (MMA M): one line segment along y
constexpr int kBTap = kC * kC * 2;           // 2 KB of weights per tap
constexpr int kBAll = kTaps * kBTap;         // 54 KB
constexpr int kLineRows = kTileM + 2;        // y = -1 .. 128 of a segment
constexpr int kChunkBytes = kLineRows * 16;  // one 16-byte K chunk of every row of a line
constexpr int kLineBytes = 4 * kChunkBytes;  // 8320 B
constexpr int kRing = 6;                     // positions along phi per x-plane: 3 in use, 1 freeing, 2 landing
constexpr int kSlots = 3 * kRing;            // line buffers
constexpr int kPChunk = 4;                   // tiles along phi per work item
constexpr int kSmemConv = kBAll + kSlots * kLineBytes + 128;  // + the mbarrier, tensor-memory slot, failure flag
static_assert(kSmemConv <= 227 * 1024, "the convolution's shared memory exceeds a CTA's limit");
constexpr uint32_t kWaitLimit = 1u << 22;    // mbarrier polls before giving up
constexpr unsigned kErrTimeout = 1u;

struct Dims {
    int nx, ny, np;
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// A voxel (x, y, p) and its linear index in the activation layout
// [x][phi][y] (every internal grid; the network's input and output are in
// the histogram layout [x][y][phi], converted by k_dn_transpose).
// moved(tap) is the periodic neighbour at tap = (dx + 1) 9 + (dy + 1) 3 + (dp + 1).
struct Vox {
    int x, y, p;
    __device__ __forceinline__ static Vox from_act(int a, Dims d) {
        return Vox{a / (d.ny * d.np), a % d.ny, (a / d.ny) % d.np};
    }
    __device__ __forceinline__ Vox moved(int tap, Dims d) const {
        int a = x + tap / 9 - 1, b = y + (tap / 3) % 3 - 1, c = p + tap % 3 - 1;
        a = a < 0 ? a + d.nx : (a >= d.nx ? a - d.nx : a);
        b = b < 0 ? b + d.ny : (b >= d.ny ? b - d.ny : b);
        c = c < 0 ? c + d.np : (c >= d.np ? c - d.np : c);
        return Vox{a, b, c};
    }
    __device__ __forceinline__ int act(Dims d) const { return (x * d.np + p) * d.ny + y; }
};

// ---- PTX wrappers ------------------------------------------------------
__device__ __forceinline__ void cp_async16(uint32_t dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }
__device__ __forceinline__ void mbar_init(uint32_t addr, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(addr), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory"); }
__device__ __forceinline__ bool mbar_try_wait(uint32_t addr, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(addr), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait for the completion of the phase with this parity
__device__ __forceinline__ bool mbar_wait(uint32_t addr, uint32_t parity) {
    for (uint32_t i = 0; i < kWaitLimit; ++i)
        if (mbar_try_wait(addr, parity)) return true;
    return false;
}
__device__ __forceinline__ void tc_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tmem_alloc(uint32_t slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(slot), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(ncols) : "memory");
}
// D[tmem] (+)= A[smem] * B[smem]^T, kind::f16 (BF16 operands, FP32 accumulator)
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar)
                 : "memory");
}
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
}

// shared-memory matrix descriptor: K-major, no swizzle; lbo = byte offset
// between K-adjacent core matrices, sbo = between 8-row groups
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// instruction descriptor: D FP32, A and B BF16, both K-major, N = 32, M = 128
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kC >> 3) << 17) |
                            ((uint32_t)(kTileM >> 4) << 24);

// byte offset of element (row, k) of a K-major operand block in the core-matrix layout
__host__ __device__ __forceinline__ int core_offset(int row, int k) {
    return (row >> 3) * 512 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2;
}

// MODE 0: bias + ReLU -> BF16; MODE 1: bias -> FP32; MODE 2: times ReLU'(ref) -> BF16.
// Work item = (x, y segment, kPChunk consecutive phi); ny a multiple of 128.
// Two accumulators in tensor memory (columns 0-31 and 32-63) pipeline the
// tiles of a work item: the MMAs of tile k run while the CTA's warps take
// tile k - 1's accumulator out (epilogue) and start the copies of the line
// tile k + 2 adds, two tiles ahead, into the ring slot of a line whose last
// MMAs completed before.
template <int MODE>
__global__ void __launch_bounds__(kTileM, 1) k_conv32(const __nv_bfloat16 *__restrict__ X,
                                                      const uint8_t *__restrict__ Wpacked,
                                                      const float *__restrict__ bias,
                                                      const __nv_bfloat16 *__restrict__ ref, void *__restrict__ Y,
                                                      Dims d, int nitems, unsigned *__restrict__ err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t *sB = smem;
    uint8_t *sL = smem + kBAll;
    uint64_t *mbar = reinterpret_cast<uint64_t *>(sL + kSlots * kLineBytes);  // one per accumulator
    uint32_t *tslot = reinterpret_cast<uint32_t *>(mbar + 2);
    volatile int *sfail = reinterpret_cast<volatile int *>(tslot + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    for (int i = tid; i < kBAll / 16; i += kTileM)
        reinterpret_cast<uint4 *>(sB)[i] = reinterpret_cast<const uint4 *>(Wpacked)[i];
    if (tid == 0) {
        mbar_init(smem_u32(mbar), 1);
        mbar_init(smem_u32(mbar + 1), 1);
        *sfail = 0;
        fence_mbar_init();
    }
    if (warp == 0) tmem_alloc(smem_u32(tslot), 64);
    fence_proxy_async();
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    const uint32_t tmem = *tslot;
    const uint32_t sL0 = smem_u32(sL), sB0 = smem_u32(sB);
    const int nseg = d.ny / kTileM, npc = (d.np + kPChunk - 1) / kPChunk;
    uint32_t phase0 = 0, phase1 = 0;

    for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
        const int pc = item % npc, ys = (item / npc) % nseg, x = item / (npc * nseg);
        const int p0 = pc * kPChunk, pcount = min(kPChunk, d.np - p0), y0 = ys * kTileM;
        // line (x + dx, p0 + q - 1) of this segment, rows y0 - 1 .. y0 + 128, into slot (dx + 1) kRing + q % kRing
        auto load_line = [&](int dx, int q) {
            int xl = x + dx, pl = p0 + q - 1;
            xl = xl < 0 ? xl + d.nx : (xl >= d.nx ? xl - d.nx : xl);
            pl = ((pl % d.np) + d.np) % d.np;
            const __nv_bfloat16 *line = X + (size_t)(xl * d.np + pl) * d.ny * kC;
            const uint32_t dst0 = sL0 + (uint32_t)(((dx + 1) * kRing + q % kRing) * kLineBytes);
            for (int e = tid; e < kLineRows * 4; e += kTileM) {
                const int r = e >> 2, j = e & 3;
                int yl = y0 + r - 1;
                yl = yl < 0 ? yl + d.ny : (yl >= d.ny ? yl - d.ny : yl);
                cp_async16(dst0 + j * kChunkBytes + r * 16, line + (size_t)yl * kC + j * 8);
            }
        };
        // accumulator of tile kt -> bias / ReLU -> Y (every thread one row)
        auto epilogue = [&](int kt) -> bool {
            const int a = kt & 1;
            if (!mbar_wait(smem_u32(mbar + a), a ? phase1 : phase0)) return false;
            if (a) phase1 ^= 1u;
            else phase0 ^= 1u;
            tc_after_sync();
            uint32_t r[32];
            tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(32 * a), r);
            const size_t vo = (size_t)((x * d.np + p0 + kt) * d.ny + y0 + warp * 32 + lane);  // this thread's row
            if (MODE == 1) {
                float4 *out = reinterpret_cast<float4 *>(reinterpret_cast<float *>(Y) + vo * kC);
#pragma unroll
                for (int q = 0; q < 8; ++q)
                    out[q] = make_float4(__uint_as_float(r[4 * q]) + bias[4 * q],
                                         __uint_as_float(r[4 * q + 1]) + bias[4 * q + 1],
                                         __uint_as_float(r[4 * q + 2]) + bias[4 * q + 2],
                                         __uint_as_float(r[4 * q + 3]) + bias[4 * q + 3]);
            } else {
                uint32_t packed[16];
#pragma unroll
                for (int q = 0; q < 16; ++q) {
                    float a0 = __uint_as_float(r[2 * q]), b0 = __uint_as_float(r[2 * q + 1]);
                    if (MODE == 0) {
                        a0 = fmaxf(a0 + bias[2 * q], 0.f);
                        b0 = fmaxf(b0 + bias[2 * q + 1], 0.f);
                    } else {
                        const __nv_bfloat16 *rr = ref + vo * kC;
                        a0 = __bfloat162float(rr[2 * q]) > 0.f ? a0 : 0.f;
                        b0 = __bfloat162float(rr[2 * q + 1]) > 0.f ? b0 : 0.f;
                    }
                    __nv_bfloat162 h = __floats2bfloat162_rn(a0, b0);
                    packed[q] = *reinterpret_cast<uint32_t *>(&h);
                }
                uint4 *out = reinterpret_cast<uint4 *>(reinterpret_cast<__nv_bfloat16 *>(Y) + vo * kC);
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    out[q] = make_uint4(packed[4 * q], packed[4 * q + 1], packed[4 * q + 2], packed[4 * q + 3]);
            }
            return true;
        };
        for (int q = 0; q < 3; ++q)
            for (int dx = -1; dx <= 1; ++dx) load_line(dx, q);
        cp_async_commit();
        if (3 <= pcount + 1)
            for (int dx = -1; dx <= 1; ++dx) load_line(dx, 3);
        cp_async_commit();
        int k = 0;
        for (; k < pcount; ++k) {
            // the line tile k + 2 adds goes into the slot of line k - 2, whose
            // last MMAs (tile k - 2) completed before tile k - 2's epilogue
            if (k + 4 <= pcount + 1)
                for (int dx = -1; dx <= 1; ++dx) load_line(dx, k + 4);
            cp_async_commit();
            cp_async_wait<2>();  // the lines of tile k have landed
            fence_proxy_async();
            __syncthreads();
            if (*sfail) break;
            if (tid == 0) {
                tc_after_sync();
                const uint32_t dacc = tmem + (uint32_t)(32 * (k & 1));
                uint32_t acc = 0;
                for (int dx = -1; dx <= 1; ++dx)
                    for (int dp = -1; dp <= 1; ++dp) {
                        const uint32_t line = sL0 + (uint32_t)(((dx + 1) * kRing + (k + 1 + dp) % kRing) * kLineBytes);
#pragma unroll
                        for (int dy = -1; dy <= 1; ++dy) {
                            const int tap = (dx + 1) * 9 + (dy + 1) * 3 + (dp + 1);
#pragma unroll
                            for (int kk = 0; kk < 2; ++kk) {
                                const uint64_t ad = smem_desc(line + kk * 2 * kChunkBytes + (1 + dy) * 16, kChunkBytes, 128);
                                const uint64_t bd = smem_desc(sB0 + tap * kBTap + kk * 256, 128, 512);
                                mma_bf16(dacc, ad, bd, kIdesc, acc);
                                acc = 1;
                            }
                        }
                    }
                mma_commit(smem_u32(mbar + (k & 1)));
            }
            // tile k - 1 leaves its accumulator while tile k's MMAs run
            if (k > 0 && !epilogue(k - 1)) *sfail = 1;
            // every thread's tensor-memory reads finish before tile k + 1's MMAs overwrite that accumulator
            tc_before_sync();
            __syncthreads();
        }
        if (*sfail) break;
        if (pcount > 0) {
            if (!epilogue(pcount - 1)) *sfail = 1;
            tc_before_sync();
            __syncthreads();
            if (*sfail) break;
        }
    }
    if (*sfail && tid == 0) atomicOr(err, kErrTimeout);
    cp_async_wait<0>();
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    if (warp == 0) tmem_dealloc(tmem, 64);
}

// FP32 weights W[tap][n][k] -> BF16 in the K-major core-matrix layout of the
// B operand, one 2 KB block per tap.  MIRROR: block t holds W[26 - t][k][n]
// (the weights of the backward-data convolution).
template <bool MIRROR>
__global__ void k_pack_weights(const float *__restrict__ W, uint8_t *__restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kTaps * kC * kC) return;
    const int t = i / (kC * kC), n = (i / kC) % kC, k = i % kC;
    const float w = MIRROR ? W[((kTaps - 1 - t) * kC + k) * kC + n] : W[(t * kC + n) * kC + k];
    *reinterpret_cast<__nv_bfloat16 *>(out + t * kBTap + core_offset(n, k)) = __float2bfloat16_rn(w);
}

int g_sms = 0;

// work items of the convolution: (x, y segment of 128, kPChunk positions along phi)
int conv_items(Dims d) { return d.nx * (d.ny / kTileM) * ((d.np + kPChunk - 1) / kPChunk); }

// ---- the network's CUDA-core layers -----------------------------------
// Parameters (FP32, one array): w_in[27][32], b_in[32], w2[27][32][32],
// b2[32], w3[27][32][32], b3[32], w_out[27][32], b_out.
constexpr int kOffWin = 0, kOffBin = kOffWin + kTaps * kC, kOffW2 = kOffBin + kC, kOffB2 = kOffW2 + kTaps * kC * kC,
              kOffW3 = kOffB2 + kC, kOffB3 = kOffW3 + kTaps * kC * kC, kOffWout = kOffB3 + kC,
              kOffBout = kOffWout + kTaps * kC, kParams = kOffBout + 1;

__device__ __forceinline__ void store_bf16x32(__nv_bfloat16 *dst, const float (&a)[32]) {
    uint32_t q[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        __nv_bfloat162 h = __floats2bfloat162_rn(a[2 * i], a[2 * i + 1]);
        q[i] = *reinterpret_cast<uint32_t *>(&h);
    }
    uint4 *o = reinterpret_cast<uint4 *>(dst);
#pragma unroll
    for (int i = 0; i < 4; ++i) o[i] = make_uint4(q[4 * i], q[4 * i + 1], q[4 * i + 2], q[4 * i + 3]);
}
__device__ __forceinline__ void load_bf16x32(const __nv_bfloat16 *src, float (&a)[32]) {
    const uint4 *s = reinterpret_cast<const uint4 *>(src);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const uint4 u = s[i];
        const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const __nv_bfloat162 h = *reinterpret_cast<const __nv_bfloat162 *>(&w[j]);
            a[8 * i + 2 * j] = __low2float(h);
            a[8 * i + 2 * j + 1] = __high2float(h);
        }
    }
}

// FP32 grids between the histogram layout [x][y][phi] and the activation
// layout [x][phi][y]: per plane x a transpose in 32 x 32 tiles
template <bool TO_ACT>
__global__ void k_dn_transpose(const float *__restrict__ src, float *__restrict__ dst, Dims d) {
    __shared__ float t[32][33];
    const int R = TO_ACT ? d.ny : d.np, Cn = TO_ACT ? d.np : d.ny;  // source rows, columns
    const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
    const float *sp = src + (size_t)blockIdx.z * d.ny * d.np;
    float *op = dst + (size_t)blockIdx.z * d.ny * d.np;
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int r = r0 + i, c = c0 + threadIdx.x;
        if (r < R && c < Cn) t[i][threadIdx.x] = sp[(size_t)r * Cn + c];
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int c = c0 + i, r = r0 + threadIdx.x;
        if (c < Cn && r < R) op[(size_t)c * R + r] = t[threadIdx.x][i];
    }
}

// ---- tiled input and output layers -------------------------------------
// A CTA of 128 threads takes the tile x = x0, phi = p0, p0 + 1, y = y0 ..
// y0 + 127 (256 voxels, 2 per thread: the same y, both phi rows) and stages
// its periodic halo (x0 +- 1, p0 - 1 .. p0 + 2, y0 - 1 .. y0 + 128) in
// shared memory once; the 27 taps then read shared memory, and each staged
// row serves both voxels of its thread.  Activation rows (32 channels, 64 B)
// are stored with their four 16-byte chunks permuted by (row >> 1) & 3, so
// that 8 consecutive rows read by one phase of a 128-bit load fall in 8
// distinct bank groups.
constexpr int kTileY = 128, kTileP = 2, kHaloY = kTileY + 2, kHaloP = kTileP + 2;
constexpr int kOutSmem = 3 * kHaloP * kHaloY * 64;  // bf16 rows of the output layer's input

__device__ __forceinline__ int wrap_idx(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }
__device__ __forceinline__ int tile_chunk(int row, int k) { return k ^ ((row >> 1) & 3); }

// tile coordinates of the CTA: blockIdx.x over (x, phi pairs, y chunks)
__device__ __forceinline__ void tile_origin(Dims d, int &x0, int &p0, int &y0) {
    const int ny_t = d.ny / kTileY, np_t = (d.np + kTileP - 1) / kTileP;
    int b = blockIdx.x;
    y0 = (b % ny_t) * kTileY;
    b /= ny_t;
    p0 = (b % np_t) * kTileP;
    x0 = b / np_t;
}

// input layer 1 -> 32 channels, ReLU: A1[v] = ReLU(b_in + sum_tap w_in[tap] x[nbr(v, tap)])
// (x in the activation layout)
__global__ void __launch_bounds__(128) k_dn_in_tiled(const float *__restrict__ x, const float *__restrict__ P,
                                                     __nv_bfloat16 *__restrict__ A1, Dims d) {
    __shared__ __align__(16) float sw[kTaps * kC + kC];
    __shared__ float sx[3][kHaloP][kHaloY];
    int x0, p0, y0;
    tile_origin(d, x0, p0, y0);
    for (int i = threadIdx.x; i < kTaps * kC + kC; i += blockDim.x) sw[i] = P[kOffWin + i];
    for (int i = threadIdx.x; i < 3 * kHaloP * kHaloY; i += blockDim.x) {
        const int ys = i % kHaloY, ip = (i / kHaloY) % kHaloP, ix = i / (kHaloY * kHaloP);
        const int gx = wrap_idx(x0 + ix - 1, d.nx), gp = wrap_idx(p0 + ip - 1, d.np), gy = wrap_idx(y0 + ys - 1, d.ny);
        sx[ix][ip][ys] = x[((size_t)gx * d.np + gp) * d.ny + gy];
    }
    __syncthreads();
    const int ty = threadIdx.x;
    float a0[32], a1[32];
#pragma unroll
    for (int c = 0; c < kC; ++c) a0[c] = a1[c] = sw[kTaps * kC + c];
    for (int t = 0; t < kTaps; ++t) {
        const int dx = t / 9, dy = (t / 3) % 3, dp = t % 3;  // tap = (dx+1) 9 + (dy+1) 3 + (dp+1)
        const float x0v = sx[dx][dp][ty + dy], x1v = sx[dx][dp + 1][ty + dy];
        const float4 *w4 = reinterpret_cast<const float4 *>(sw + t * kC);
#pragma unroll
        for (int c4 = 0; c4 < kC / 4; ++c4) {
            const float4 w = w4[c4];
            a0[4 * c4] = fmaf(w.x, x0v, a0[4 * c4]);
            a0[4 * c4 + 1] = fmaf(w.y, x0v, a0[4 * c4 + 1]);
            a0[4 * c4 + 2] = fmaf(w.z, x0v, a0[4 * c4 + 2]);
            a0[4 * c4 + 3] = fmaf(w.w, x0v, a0[4 * c4 + 3]);
            a1[4 * c4] = fmaf(w.x, x1v, a1[4 * c4]);
            a1[4 * c4 + 1] = fmaf(w.y, x1v, a1[4 * c4 + 1]);
            a1[4 * c4 + 2] = fmaf(w.z, x1v, a1[4 * c4 + 2]);
            a1[4 * c4 + 3] = fmaf(w.w, x1v, a1[4 * c4 + 3]);
        }
    }
#pragma unroll
    for (int c = 0; c < kC; ++c) {
        a0[c] = fmaxf(a0[c], 0.f);
        a1[c] = fmaxf(a1[c], 0.f);
    }
    const int y = y0 + ty;
    store_bf16x32(A1 + (((size_t)x0 * d.np + p0) * d.ny + y) * kC, a0);
    if (p0 + 1 < d.np) store_bf16x32(A1 + (((size_t)x0 * d.np + p0 + 1) * d.ny + y) * kC, a1);
}

// output layer 32 -> 1 with the residual: y[v] = x[v] + b_out + sum_tap w_out[tap] . A3[nbr(v, tap)]
// (x and y in the activation layout)
__global__ void __launch_bounds__(128) k_dn_out_tiled(const __nv_bfloat16 *__restrict__ A3,
                                                      const float *__restrict__ x, const float *__restrict__ P,
                                                      float *__restrict__ y, Dims d) {
    extern __shared__ __align__(16) unsigned char dn_out_smem[];
    float *sw = reinterpret_cast<float *>(dn_out_smem + kOutSmem);
    int x0, p0, y0;
    tile_origin(d, x0, p0, y0);
    const uint32_t base = smem_u32(dn_out_smem);
    for (int i = threadIdx.x; i < 3 * kHaloP * kHaloY * 4; i += blockDim.x) {
        const int k = i & 3, r = i >> 2;  // 16-byte chunk k of staged row r
        const int ys = r % kHaloY, ip = (r / kHaloY) % kHaloP, ix = r / (kHaloY * kHaloP);
        const int gx = wrap_idx(x0 + ix - 1, d.nx), gp = wrap_idx(p0 + ip - 1, d.np), gy = wrap_idx(y0 + ys - 1, d.ny);
        cp_async16(base + (uint32_t)(r * 64 + tile_chunk(ys, k) * 16),
                   A3 + (((size_t)gx * d.np + gp) * d.ny + gy) * kC + 8 * k);
    }
    cp_async_commit();
    for (int i = threadIdx.x; i < kTaps * kC + 1; i += blockDim.x) sw[i] = P[kOffWout + i];
    cp_async_wait<0>();
    __syncthreads();
    const int ty = threadIdx.x;
    // one partial sum per 8-channel chunk and voxel: 8 independent FMA chains per thread
    float acc0[4] = {0.f, 0.f, 0.f, 0.f}, acc1[4] = {0.f, 0.f, 0.f, 0.f};
    for (int dx = 0; dx < 3; ++dx) {
        for (int dy = 0; dy < 3; ++dy) {
            const int ys = ty + dy;
#pragma unroll
            for (int ip = 0; ip < kHaloP; ++ip) {
                // staged row (dx, ip, ys) is tap (dx, dy, ip) of voxel p0 and tap (dx, dy, ip - 1) of voxel p0 + 1
                const int r = (dx * kHaloP + ip) * kHaloY + ys;
                const float4 *w0 = reinterpret_cast<const float4 *>(sw + (dx * 9 + dy * 3 + ip) * kC);
                const float4 *w1 = reinterpret_cast<const float4 *>(sw + (dx * 9 + dy * 3 + ip - 1) * kC);
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const uint4 u = *reinterpret_cast<const uint4 *>(dn_out_smem + r * 64 + tile_chunk(ys, k) * 16);
                    const float v[8] = {__uint_as_float(u.x << 16), __uint_as_float(u.x & 0xFFFF0000u),
                                        __uint_as_float(u.y << 16), __uint_as_float(u.y & 0xFFFF0000u),
                                        __uint_as_float(u.z << 16), __uint_as_float(u.z & 0xFFFF0000u),
                                        __uint_as_float(u.w << 16), __uint_as_float(u.w & 0xFFFF0000u)};
                    if (ip < 3) {
                        const float4 a = w0[2 * k], b = w0[2 * k + 1];
                        float t = acc0[k];
                        t = fmaf(a.x, v[0], t); t = fmaf(a.y, v[1], t); t = fmaf(a.z, v[2], t); t = fmaf(a.w, v[3], t);
                        t = fmaf(b.x, v[4], t); t = fmaf(b.y, v[5], t); t = fmaf(b.z, v[6], t); t = fmaf(b.w, v[7], t);
                        acc0[k] = t;
                    }
                    if (ip > 0) {
                        const float4 a = w1[2 * k], b = w1[2 * k + 1];
                        float t = acc1[k];
                        t = fmaf(a.x, v[0], t); t = fmaf(a.y, v[1], t); t = fmaf(a.z, v[2], t); t = fmaf(a.w, v[3], t);
                        t = fmaf(b.x, v[4], t); t = fmaf(b.y, v[5], t); t = fmaf(b.z, v[6], t); t = fmaf(b.w, v[7], t);
                        acc1[k] = t;
                    }
                }
            }
        }
    }
    const float bo = sw[kTaps * kC];
    const size_t v0 = ((size_t)x0 * d.np + p0) * d.ny + y0 + ty;
    y[v0] = x[v0] + ((acc0[0] + acc0[1]) + (acc0[2] + acc0[3])) + bo;
    if (p0 + 1 < d.np) y[v0 + d.ny] = x[v0 + d.ny] + ((acc1[0] + acc1[1]) + (acc1[2] + acc1[3])) + bo;
}

// mean-square loss against the target and its gradient dy = 2 (y - t) / V;
// sums (y - t)^2 / V and dy (the output bias gradient) in FP64
__global__ void k_dn_loss(const float *__restrict__ y, const float *__restrict__ t, float *__restrict__ dy, int nvox,
                          double *__restrict__ sums, float *__restrict__ db_out) {
    double l = 0.0, g = 0.0;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nvox; v += gridDim.x * blockDim.x) {
        const float r = y[v] - t[v];
        const float gv = 2.f * r / (float)nvox;
        dy[v] = gv;
        l += (double)(r * r);
        g += (double)gv;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        l += __shfl_xor_sync(0xffffffffu, l, o);
        g += __shfl_xor_sync(0xffffffffu, g, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&sums[0], l / (double)nvox);
        if (db_out) atomicAdd(db_out, (float)g);
    }
}

// the loss with the angular-moment term: per cell (x, y) the residual
// r = y - t over phi has the second harmonic c2 = sum_k r_k cos 2 phi_k,
// s2 = sum_k r_k sin 2 phi_k (phi_k the bin centres).  In the plane the active
// stress of a cell, and with it the flow, depends on the cell's orientation
// distribution only through its density and this harmonic, and the Oseen
// projection removes the density's part, so the flow error of a denoised
// histogram is the error of this harmonic.  The loss is
//     mean_v r^2 + w * sum_cells (c2^2 + s2^2) / V
// (for white noise both terms are alike at w = 1), its gradient
//     dy_k = 2 / V * (r_k + w (c2 cos 2 phi_k + s2 sin 2 phi_k)).
// One thread per cell; the layout is [x][phi][y], so consecutive threads
// read consecutive y.
__global__ void k_dn_loss_moment(const float *__restrict__ y, const float *__restrict__ t, float *__restrict__ dy,
                                 Dims d, float w, double *__restrict__ sums, float *__restrict__ db_out) {
    extern __shared__ float cs[];  // cos 2 phi_k, then sin 2 phi_k
    for (int k = threadIdx.x; k < d.np; k += blockDim.x) {
        float sn, cn;
        sincospif((2.f * (float)k + 1.f) * 2.f / (float)d.np, &sn, &cn);  // 2 phi_k / pi
        cs[k] = cn;
        cs[d.np + k] = sn;
    }
    __syncthreads();
    const int ncell = d.nx * d.ny;
    const float inv_v = 1.f / (float)((long long)ncell * d.np);
    double l = 0.0, g = 0.0;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += gridDim.x * blockDim.x) {
        const int x = c / d.ny, yy = c - x * d.ny;
        const size_t base = (size_t)x * d.np * d.ny + yy;
        float c2 = 0.f, s2 = 0.f;
        for (int k = 0; k < d.np; ++k) {
            const size_t v = base + (size_t)k * d.ny;
            const float r = y[v] - t[v];
            c2 = fmaf(cs[k], r, c2);
            s2 = fmaf(cs[d.np + k], r, s2);
        }
        const float mc = w * c2, ms = w * s2;
        for (int k = 0; k < d.np; ++k) {
            const size_t v = base + (size_t)k * d.ny;
            const float r = y[v] - t[v];
            const float gv = 2.f * inv_v * (r + fmaf(mc, cs[k], ms * cs[d.np + k]));
            dy[v] = gv;
            l += (double)(r * r);
            g += (double)gv;
        }
        l += (double)w * ((double)c2 * c2 + (double)s2 * s2);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        l += __shfl_xor_sync(0xffffffffu, l, o);
        g += __shfl_xor_sync(0xffffffffu, g, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&sums[0], l * (double)inv_v);
        if (db_out) atomicAdd(db_out, (float)g);
    }
}

// backward of the output layer into its input: dZ3[u][c] = (sum_tap
// w_out[tap][c] dy[nbr(u, 26 - tap)]) * (A3[u][c] > 0)
__global__ void __launch_bounds__(128) k_dn_out_bwd(const float *__restrict__ dy, const float *__restrict__ P,
                                                    const __nv_bfloat16 *__restrict__ A3,
                                                    __nv_bfloat16 *__restrict__ dZ3, Dims d, int nvox) {
    __shared__ float sw[kTaps * kC];
    for (int i = threadIdx.x; i < kTaps * kC; i += blockDim.x) sw[i] = P[kOffWout + i];
    __syncthreads();
    const int u = blockIdx.x * blockDim.x + threadIdx.x;  // activation index
    if (u >= nvox) return;
    const Vox vx = Vox::from_act(u, d);
    float g[32];
#pragma unroll
    for (int c = 0; c < kC; ++c) g[c] = 0.f;
    for (int t = 0; t < kTaps; ++t) {
        const float dv = dy[vx.moved(kTaps - 1 - t, d).act(d)];
#pragma unroll
        for (int c = 0; c < kC; ++c) g[c] = fmaf(sw[t * kC + c], dv, g[c]);
    }
    float a[32];
    load_bf16x32(A3 + (size_t)u * kC, a);
#pragma unroll
    for (int c = 0; c < kC; ++c) g[c] = a[c] > 0.f ? g[c] : 0.f;
    store_bf16x32(dZ3 + (size_t)u * kC, g);
}

// Reduce-scatter across a warp: each lane holds v[0..31]; afterwards lane l
// holds the sum over the warp of v[l] (31 shuffles instead of 32 x 5).
__device__ __forceinline__ float warp_reduce_scatter32(float (&v)[32]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int half = 16; half >= 1; half >>= 1) {
        const bool up = (lane & half) != 0;
#pragma unroll
        for (int j = 0; j < half; ++j) {
            const float send = up ? v[j] : v[j + half];
            const float keep = up ? v[j + half] : v[j];
            v[j] = keep + __shfl_xor_sync(0xffffffffu, send, half);
        }
    }
    return v[0];
}

// Weight gradients of the 1-channel layers, one tile of 128 voxels per
// block iteration (persistent grid):
//   OUT: dW[tap][c] += sum_v dy[v] A3[nbr(v, tap)][c]   (S = A3, sv = dy)
//   IN:  dW[tap][c] += sum_v dZ1[v][c] x[nbr(v, tap)]   (S = dZ1, sv = x),
//        and db[c] += sum_v dZ1[v][c]
// Per tap the warp's 32 x 32 products are reduce-scattered to one channel
// per lane and added into the block's shared accumulator.
template <bool OUT>
__global__ void __launch_bounds__(128) k_dn_wgrad_c1(const __nv_bfloat16 *__restrict__ S, const float *__restrict__ sv,
                                                     float *__restrict__ dW, float *__restrict__ db, Dims d,
                                                     int ntiles) {
    __shared__ float acc[kTaps * kC + kC];
    const int tid = threadIdx.x, lane = tid & 31;
    for (int i = tid; i < kTaps * kC + kC; i += blockDim.x) acc[i] = 0.f;
    __syncthreads();
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int v = tile * kTileM + tid;  // activation index
        const Vox vx = Vox::from_act(v, d);
        float own[32];
        float s_own = 0.f;
        if (OUT) {
            s_own = sv[v];
        } else {
            load_bf16x32(S + (size_t)v * kC, own);
            float t[32];
#pragma unroll
            for (int c = 0; c < kC; ++c) t[c] = own[c];
            atomicAdd(&acc[kTaps * kC + lane], warp_reduce_scatter32(t));
        }
        for (int tap = 0; tap < kTaps; ++tap) {
            const Vox u = vx.moved(tap, d);
            float p[32];
            if (OUT) {
                load_bf16x32(S + (size_t)u.act(d) * kC, p);
#pragma unroll
                for (int c = 0; c < kC; ++c) p[c] *= s_own;
            } else {
                const float xs = sv[u.act(d)];
#pragma unroll
                for (int c = 0; c < kC; ++c) p[c] = own[c] * xs;
            }
            atomicAdd(&acc[tap * kC + lane], warp_reduce_scatter32(p));
        }
    }
    __syncthreads();
    for (int i = tid; i < kTaps * kC; i += blockDim.x) atomicAdd(&dW[i], acc[i]);
    if (!OUT && tid < kC) atomicAdd(&db[tid], acc[kTaps * kC + tid]);
}

// weight gradient of a 32 -> 32 layer: dW[tap][co][ci] = sum_v dZ[v][co] A[nbr(v, tap)][ci].
// Grid (27 taps, blocks over voxel tiles of 128).  A tile of dZ and the
// tap-shifted tile of A are staged in shared memory as FP32; each thread
// accumulates a 4 x 4 block of (co, ci) over a quarter of the tile's voxels.
__global__ void __launch_bounds__(256) k_dn_wgrad32(const __nv_bfloat16 *__restrict__ dZ,
                                                    const __nv_bfloat16 *__restrict__ A, float *__restrict__ dW,
                                                    float *__restrict__ db, Dims d, int ntiles) {
    __shared__ __align__(16) float sZ[kTileM][kC + 4];
    __shared__ __align__(16) float sA[kTileM][kC + 4];
    const int tap = blockIdx.x, tid = threadIdx.x;
    const int g = tid >> 6, lt = tid & 63, cb = lt >> 3, ib = lt & 7;
    float acc[4][4], bacc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
    const int r = tid >> 1, h = tid & 1;
    const bool centre = tap == kTaps / 2 && ib == 0;  // these threads also sum dZ (the bias gradient)
    for (int tile = blockIdx.y; tile < ntiles; tile += gridDim.y) {
        const int v = tile * kTileM + r;  // activation indices
        const int u = Vox::from_act(v, d).moved(tap, d).act(d);
        const uint4 *zs = reinterpret_cast<const uint4 *>(dZ + (size_t)v * kC + 16 * h);
        const uint4 *as = reinterpret_cast<const uint4 *>(A + (size_t)u * kC + 16 * h);
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const uint4 zu = zs[q], au = as[q];
            const uint32_t zw[4] = {zu.x, zu.y, zu.z, zu.w}, aw[4] = {au.x, au.y, au.z, au.w};
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const __nv_bfloat162 zh = *reinterpret_cast<const __nv_bfloat162 *>(&zw[j]);
                const __nv_bfloat162 ah = *reinterpret_cast<const __nv_bfloat162 *>(&aw[j]);
                sZ[r][16 * h + 8 * q + 2 * j] = __low2float(zh);
                sZ[r][16 * h + 8 * q + 2 * j + 1] = __high2float(zh);
                sA[r][16 * h + 8 * q + 2 * j] = __low2float(ah);
                sA[r][16 * h + 8 * q + 2 * j + 1] = __high2float(ah);
            }
        }
        __syncthreads();
#pragma unroll 4
        for (int k = g; k < kTileM; k += 4) {
            const float4 z = *reinterpret_cast<const float4 *>(&sZ[k][4 * cb]);
            const float4 a = *reinterpret_cast<const float4 *>(&sA[k][4 * ib]);
            const float zz[4] = {z.x, z.y, z.z, z.w}, aa[4] = {a.x, a.y, a.z, a.w};
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(zz[i], aa[j], acc[i][j]);
            if (centre) {
#pragma unroll
                for (int i = 0; i < 4; ++i) bacc[i] += zz[i];
            }
        }
        __syncthreads();
    }
    // the four voxel groups' partial sums, then one atomic per (co, ci)
    float *red = &sZ[0][0];  // 4 x 64 x 16 floats fit in sZ
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) red[(g * 64 + lt) * 16 + 4 * i + j] = acc[i][j];
    __syncthreads();
    for (int o = tid; o < kC * kC; o += blockDim.x) {
        const int co = o >> 5, ci = o & 31;
        const int l = (co >> 2) * 8 + (ci >> 2), e = (co & 3) * 4 + (ci & 3);
        const float s = red[(0 * 64 + l) * 16 + e] + red[(1 * 64 + l) * 16 + e] + red[(2 * 64 + l) * 16 + e] +
                        red[(3 * 64 + l) * 16 + e];
        atomicAdd(&dW[(tap * kC + co) * kC + ci], s);
    }
    if (centre) {
#pragma unroll
        for (int i = 0; i < 4; ++i) atomicAdd(&db[4 * cb + i], bacc[i]);
    }
}

// Adam (Kingma and Ba, 2015) on the FP32 parameters
__global__ void k_dn_adam(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                          float *__restrict__ s, int n, float gscale, float lr, float b1, float b2, float eps, float c1,
                          float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i] * gscale;
    const float mi = b1 * m[i] + (1.f - b1) * gi, si = b2 * s[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    s[i] = si;
    p[i] -= lr * (mi / c1) / (sqrtf(si / c2) + eps);
}

}  // namespace

extern "C" int ss_dn_conv32(const void *x, const float *w, const float *bias, const void *ref, void *y,
                            uint32_t nx, uint32_t ny, uint32_t np, uint32_t mode, void *stream) {
    char buf[256];
    if (!x || !w || !y || (mode != 2 && !bias) || (mode == 2 && !ref) || mode > 2 || nx < 1 || ny < 1 || np < 1 ||
        ny % kTileM != 0 || (unsigned long long)nx * ny * np > (1ull << 27)) {
        ss::record_error("ss_dn_conv32: null pointer, mode > 2, or ny not a positive multiple of 128");
        return SS_ERR_INVALID_ARGUMENT;
    }
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaSuccess;
    if (!g_sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
        if (g_sms <= 0) g_sms = 1;
        cudaFuncSetAttribute(k_conv32<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemConv);
        cudaFuncSetAttribute(k_conv32<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemConv);
        cudaFuncSetAttribute(k_conv32<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemConv);
    }
    uint8_t *packed = nullptr;
    unsigned *derr = nullptr;
    e = cudaMallocAsync((void **)&packed, kBAll, s);
    if (e == cudaSuccess) e = cudaMallocAsync((void **)&derr, sizeof(unsigned), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(derr, 0, sizeof(unsigned), s);
    if (e == cudaSuccess) {
        const int nw = kTaps * kC * kC;
        if (mode == 2) k_pack_weights<true><<<(nw + 255) / 256, 256, 0, s>>>(w, packed);
        else k_pack_weights<false><<<(nw + 255) / 256, 256, 0, s>>>(w, packed);
        Dims d{(int)nx, (int)ny, (int)np};
        const int items = conv_items(d), grid = items < g_sms ? items : g_sms;
        const __nv_bfloat16 *X = reinterpret_cast<const __nv_bfloat16 *>(x);
        const __nv_bfloat16 *R = reinterpret_cast<const __nv_bfloat16 *>(ref);
        if (mode == 0) k_conv32<0><<<grid, kTileM, kSmemConv, s>>>(X, packed, bias, R, y, d, items, derr);
        else if (mode == 1) k_conv32<1><<<grid, kTileM, kSmemConv, s>>>(X, packed, bias, R, y, d, items, derr);
        else k_conv32<2><<<grid, kTileM, kSmemConv, s>>>(X, packed, bias, R, y, d, items, derr);
        e = cudaGetLastError();
    }
    unsigned herr = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, derr, sizeof herr, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFreeAsync(packed, s);
    cudaFreeAsync(derr, s);
    if (e != cudaSuccess) {
        snprintf(buf, sizeof buf, "ss_dn_conv32: %s", cudaGetErrorString(e));
        ss::record_error(buf);
        return SS_ERR_CUDA;
    }
    if (herr) {
        ss::record_error("ss_dn_conv32: an mbarrier wait timed out");
        return SS_ERR_CUDA;
    }
    return SS_OK;
}

// Training data: the normalised histogram (mean 1 per bin) of n particles
// drawn from the production workload's initial condition family: density
// proportional to 1 + amp sin(2 pi s + phase) along one axis (s = position
// / box edge), uniform along the other and in phi.  The profile is sampled
// by inverting its CDF with FP32 Newton steps; Philox keyed by seed, counter
// = particle index.  Each particle adds nbins / n to its bin.
__global__ void k_dn_sample_hist(int nx, int ny, int np, unsigned long long n, float amp, float phase, int axis,
                                 unsigned long long seed, float w, float *__restrict__ hist) {
    const uint2 key = make_uint2((uint32_t)seed, (uint32_t)(seed >> 32));
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        const uint4 r = ss::philox4x32_10(make_uint4((uint32_t)i, (uint32_t)(i >> 32), 0x5EED0000u, 7u), key);
        const float u = (float)(r.x >> 8) * 0x1p-24f, u2 = (float)(r.y >> 8) * 0x1p-24f,
                    u3 = (float)(r.z >> 8) * 0x1p-24f;
        // F(s) = s - amp / (2 pi) (cos(2 pi s + phase) - cos(phase)) = u, F' = 1 + amp sin(2 pi s + phase)
        float sv = u;
        const float c0 = cosf(phase), k = amp * 0.15915494309189535f;
#pragma unroll
        for (int it = 0; it < 4; ++it) {
            float sn, cs;
            sincosf(6.283185307179586f * sv + phase, &sn, &cs);
            sv -= (sv - k * (cs - c0) - u) / (1.f + amp * sn);
        }
        sv = sv - floorf(sv);
        const int na = axis == 0 ? nx : ny, nb = axis == 0 ? ny : nx;
        int ia = (int)(sv * (float)na), ib = (int)(u2 * (float)nb), ip = (int)(u3 * (float)np);
        ia = ia < 0 ? 0 : (ia >= na ? na - 1 : ia);
        ib = ib >= nb ? nb - 1 : ib;
        ip = ip >= np ? np - 1 : ip;
        const int ix = axis == 0 ? ia : ib, iy = axis == 0 ? ib : ia;
        atomicAdd(hist + ((size_t)ix * ny + iy) * np + ip, w);
    }
}

// ---------------------------------------------------------------------------
// host object
// ---------------------------------------------------------------------------
struct ss_dn {
    Dims d{};
    int nvox = 0, ntiles = 0, sms = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int device = 0;
    // dy, yb, xa, ta: FP32 grids in the activation layout
    float *P = nullptr, *G = nullptr, *M = nullptr, *S = nullptr, *dy = nullptr, *yb = nullptr, *xa = nullptr,
          *ta = nullptr;
    uint8_t *Wp2 = nullptr, *Wp3 = nullptr, *Wm2 = nullptr, *Wm3 = nullptr;
    __nv_bfloat16 *A1 = nullptr, *A2 = nullptr, *A3 = nullptr, *D1 = nullptr, *D2 = nullptr;
    double *sums = nullptr;
    unsigned *err = nullptr;
    long long adam_t = 0;
    uint64_t launches = 0;
    float moment_weight = 0.f;  // w of the angular-moment term of the loss (k_dn_loss_moment); 0: mean-square only
};

namespace {

int dnfail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    ss::record_error(buf);
    return code;
}
#define DCK(call)                                                                                    \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess) return dnfail(SS_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

void conv_attrs() {
    static bool done = false;
    if (done) return;
    cudaFuncSetAttribute(k_conv32<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemConv);
    cudaFuncSetAttribute(k_conv32<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemConv);
    cudaFuncSetAttribute(k_conv32<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemConv);
    cudaFuncSetAttribute(k_dn_out_tiled, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         kOutSmem + (kTaps * kC + 4) * (int)sizeof(float));
    done = true;
}

template <int MODE>
void launch_conv(ss_dn *n, const __nv_bfloat16 *X, const uint8_t *W, const float *bias, const __nv_bfloat16 *ref,
                 void *Y, cudaStream_t s) {
    const int items = conv_items(n->d), grid = items < n->sms ? items : n->sms;
    k_conv32<MODE><<<grid, kTileM, kSmemConv, s>>>(X, W, bias, ref, Y, n->d, items, n->err);
}

void pack_all(ss_dn *n, cudaStream_t s) {
    const int nw = kTaps * kC * kC, b = (nw + 255) / 256;
    k_pack_weights<false><<<b, 256, 0, s>>>(n->P + kOffW2, n->Wp2);
    k_pack_weights<false><<<b, 256, 0, s>>>(n->P + kOffW3, n->Wp3);
    k_pack_weights<true><<<b, 256, 0, s>>>(n->P + kOffW2, n->Wm2);
    k_pack_weights<true><<<b, 256, 0, s>>>(n->P + kOffW3, n->Wm3);
    n->launches += 4;
}

template <bool TO_ACT>
void transpose(ss_dn *n, const float *src, float *dst, cudaStream_t s) {
    const int R = TO_ACT ? n->d.ny : n->d.np, Cn = TO_ACT ? n->d.np : n->d.ny;
    k_dn_transpose<TO_ACT><<<dim3((Cn + 31) / 32, (R + 31) / 32, n->d.nx), dim3(32, 8), 0, s>>>(src, dst, n->d);
}

// the network on x (histogram layout), output ya in the activation layout
void enqueue_forward_act(ss_dn *n, const float *x, float *ya, cudaStream_t s) {
    transpose<true>(n, x, n->xa, s);
    const unsigned tiles = (unsigned)(n->d.nx * ((n->d.np + kTileP - 1) / kTileP) * (n->d.ny / kTileY));
    k_dn_in_tiled<<<tiles, 128, 0, s>>>(n->xa, n->P, n->A1, n->d);
    launch_conv<0>(n, n->A1, n->Wp2, n->P + kOffB2, nullptr, n->A2, s);
    launch_conv<0>(n, n->A2, n->Wp3, n->P + kOffB3, nullptr, n->A3, s);
    k_dn_out_tiled<<<tiles, 128, kOutSmem + (kTaps * kC + 4) * sizeof(float), s>>>(n->A3, n->xa, n->P, ya, n->d);
    n->launches += 5;
}

void enqueue_forward(ss_dn *n, const float *x, float *y, cudaStream_t s) {
    enqueue_forward_act(n, x, n->yb, s);
    transpose<false>(n, n->yb, y, s);
    n->launches += 1;
}

// loss of y against t, then the gradients of every parameter (accumulated into G)
// (after enqueue_forward_act: n->xa holds the input, ya the output, both in the activation layout)
void enqueue_backward(ss_dn *n, const float *t, const float *ya, cudaStream_t s, bool grads) {
    const unsigned b = (unsigned)((n->nvox + 127) / 128);
    transpose<true>(n, t, n->ta, s);
    if (n->moment_weight > 0.f)
        k_dn_loss_moment<<<2 * n->sms, 128, 2 * n->d.np * sizeof(float), s>>>(
            ya, n->ta, n->dy, n->d, n->moment_weight, n->sums, grads ? n->G + kOffBout : nullptr);
    else
        k_dn_loss<<<2 * n->sms, 256, 0, s>>>(ya, n->ta, n->dy, n->nvox, n->sums, grads ? n->G + kOffBout : nullptr);
    n->launches += 2;
    if (!grads) return;
    const dim3 wg(kTaps, (unsigned)(n->sms > 0 ? (4 * n->sms + kTaps - 1) / kTaps : 8));
    const unsigned pg = (unsigned)(n->ntiles < 8 * n->sms ? n->ntiles : 8 * n->sms);
    k_dn_out_bwd<<<b, 128, 0, s>>>(n->dy, n->P, n->A3, n->D1, n->d, n->nvox);
    k_dn_wgrad_c1<true><<<pg, 128, 0, s>>>(n->A3, n->dy, n->G + kOffWout, nullptr, n->d, n->ntiles);
    k_dn_wgrad32<<<wg, 256, 0, s>>>(n->D1, n->A2, n->G + kOffW3, n->G + kOffB3, n->d, n->ntiles);
    launch_conv<2>(n, n->D1, n->Wm3, nullptr, n->A2, n->D2, s);
    k_dn_wgrad32<<<wg, 256, 0, s>>>(n->D2, n->A1, n->G + kOffW2, n->G + kOffB2, n->d, n->ntiles);
    launch_conv<2>(n, n->D2, n->Wm2, nullptr, n->A1, n->D1, s);
    k_dn_wgrad_c1<false><<<pg, 128, 0, s>>>(n->D1, n->xa, n->G + kOffWin, n->G + kOffBin, n->d, n->ntiles);
    n->launches += 8;
}

int check_err(ss_dn *n) {
    unsigned h = 0;
    DCK(cudaMemcpyAsync(&h, n->err, sizeof h, cudaMemcpyDeviceToHost, n->stream));
    DCK(cudaStreamSynchronize(n->stream));
    if (h) return dnfail(SS_ERR_CUDA, "denoiser: a tensor-core convolution's mbarrier wait timed out");
    return SS_OK;
}

void destroy_dn(ss_dn *n) {
    if (!n) return;
    cudaSetDevice(n->device);
    if (n->stream) cudaStreamSynchronize(n->stream);
    cudaFree(n->P); cudaFree(n->G); cudaFree(n->M); cudaFree(n->S); cudaFree(n->dy); cudaFree(n->yb);
    cudaFree(n->xa); cudaFree(n->ta);
    cudaFree(n->Wp2); cudaFree(n->Wp3); cudaFree(n->Wm2); cudaFree(n->Wm3);
    cudaFree(n->A1); cudaFree(n->A2); cudaFree(n->A3); cudaFree(n->D1); cudaFree(n->D2);
    cudaFree(n->sums); cudaFree(n->err);
    if (n->own_stream && n->stream) cudaStreamDestroy(n->stream);
    delete n;
}

}  // namespace

extern "C" {

int ss_dn_create(uint32_t nx, uint32_t ny, uint32_t np, uint64_t seed, void *stream, ss_dn **out) {
    if (!out) return dnfail(SS_ERR_INVALID_ARGUMENT, "ss_dn_create: null output");
    *out = nullptr;
    const unsigned long long V = (unsigned long long)nx * ny * np;
    if (nx < 1 || ny < 1 || np < 1 || ny % kTileM != 0 || V > (1ull << 27))
        return dnfail(SS_ERR_INVALID_ARGUMENT,
                      "ss_dn_create: ny must be a positive multiple of 128 (at most 2^27 voxels)");
    ss_dn *n = new ss_dn();
    n->d = Dims{(int)nx, (int)ny, (int)np};
    n->nvox = (int)V;
    n->ntiles = (int)(V / kTileM);
    cudaError_t e = cudaGetDevice(&n->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&n->sms, cudaDevAttrMultiProcessorCount, n->device);
    if (e == cudaSuccess) {
        if (stream) {
            n->stream = (cudaStream_t)stream;
        } else {
            e = cudaStreamCreateWithFlags(&n->stream, cudaStreamNonBlocking);
            n->own_stream = e == cudaSuccess;
        }
    }
    auto A = [&](void **p, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc(p, bytes);
    };
    const size_t pb = (size_t)kParams * sizeof(float), ab = (size_t)V * kC * sizeof(__nv_bfloat16);
    A((void **)&n->P, pb); A((void **)&n->G, pb); A((void **)&n->M, pb); A((void **)&n->S, pb);
    A((void **)&n->dy, V * sizeof(float)); A((void **)&n->yb, V * sizeof(float));
    A((void **)&n->xa, V * sizeof(float)); A((void **)&n->ta, V * sizeof(float));
    A((void **)&n->Wp2, kBAll); A((void **)&n->Wp3, kBAll); A((void **)&n->Wm2, kBAll); A((void **)&n->Wm3, kBAll);
    A((void **)&n->A1, ab); A((void **)&n->A2, ab); A((void **)&n->A3, ab); A((void **)&n->D1, ab);
    A((void **)&n->D2, ab);
    A((void **)&n->sums, 2 * sizeof(double)); A((void **)&n->err, sizeof(unsigned));
    // He initialisation of the convolutions; the output layer starts near
    // zero so that the network starts as the identity (residual)
    std::vector<float> h(kParams, 0.f);
    std::mt19937_64 rng(seed);
    std::normal_distribution<float> nd(0.f, 1.f);
    for (int i = 0; i < kTaps * kC; ++i) h[kOffWin + i] = nd(rng) * std::sqrt(2.f / kTaps);
    for (int i = 0; i < kTaps * kC * kC; ++i) h[kOffW2 + i] = nd(rng) * std::sqrt(2.f / (kTaps * kC));
    for (int i = 0; i < kTaps * kC * kC; ++i) h[kOffW3 + i] = nd(rng) * std::sqrt(2.f / (kTaps * kC));
    for (int i = 0; i < kTaps * kC; ++i) h[kOffWout + i] = nd(rng) * 1e-3f;
    if (e == cudaSuccess) e = cudaMemcpyAsync(n->P, h.data(), pb, cudaMemcpyHostToDevice, n->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(n->M, 0, pb, n->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(n->S, 0, pb, n->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(n->err, 0, sizeof(unsigned), n->stream);
    if (e == cudaSuccess) {
        conv_attrs();
        pack_all(n, n->stream);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(n->stream);
    if (e != cudaSuccess) {
        const std::string m = cudaGetErrorString(e);
        destroy_dn(n);
        return dnfail(SS_ERR_CUDA, "ss_dn_create: %s", m.c_str());
    }
    *out = n;
    return SS_OK;
}

int ss_dn_destroy(ss_dn *n) {
    destroy_dn(n);
    return SS_OK;
}

int ss_dn_info(ss_dn *n, uint64_t *nparams, uint64_t *launches) {
    if (!n) return dnfail(SS_ERR_INVALID_ARGUMENT, "null denoiser");
    if (nparams) *nparams = (uint64_t)kParams;
    if (launches) *launches = n->launches;
    return SS_OK;
}

int ss_dn_get_params(ss_dn *n, float *host, uint64_t count) {
    if (!n || !host || count != (uint64_t)kParams)
        return dnfail(SS_ERR_INVALID_ARGUMENT, "ss_dn_get_params: null argument or count != %d", kParams);
    DCK(cudaSetDevice(n->device));
    DCK(cudaMemcpyAsync(host, n->P, (size_t)kParams * sizeof(float), cudaMemcpyDeviceToHost, n->stream));
    DCK(cudaStreamSynchronize(n->stream));
    return SS_OK;
}

int ss_dn_set_params(ss_dn *n, const float *host, uint64_t count) {
    if (!n || !host || count != (uint64_t)kParams)
        return dnfail(SS_ERR_INVALID_ARGUMENT, "ss_dn_set_params: null argument or count != %d", kParams);
    for (uint64_t i = 0; i < count; ++i)
        if (!std::isfinite(host[i])) return dnfail(SS_ERR_INVALID_ARGUMENT, "ss_dn_set_params: non-finite parameter");
    DCK(cudaSetDevice(n->device));
    DCK(cudaMemcpyAsync(n->P, host, (size_t)kParams * sizeof(float), cudaMemcpyHostToDevice, n->stream));
    pack_all(n, n->stream);
    DCK(cudaGetLastError());
    DCK(cudaStreamSynchronize(n->stream));
    return SS_OK;
}

int ss_dn_forward(ss_dn *n, const float *x, float *y) {
    if (!n || !x || !y) return dnfail(SS_ERR_INVALID_ARGUMENT, "ss_dn_forward: null argument");
    DCK(cudaSetDevice(n->device));
    enqueue_forward(n, x, y, n->stream);
    DCK(cudaGetLastError());
    return check_err(n);
}

int ss_dn_set_loss(ss_dn *n, float moment_weight) {
    if (!n || !(moment_weight >= 0.f) || !std::isfinite(moment_weight))
        return dnfail(SS_ERR_INVALID_ARGUMENT, "ss_dn_set_loss: null network or moment weight not finite and >= 0");
    n->moment_weight = moment_weight;
    return SS_OK;
}

// batch samples [batch][V] (DEVICE): loss averaged over the batch; with
// lr > 0 one Adam step on the batch-mean gradient
int ss_dn_train(ss_dn *n, const float *x, const float *t, uint32_t batch, float lr, double *loss) {
    if (!n || !x || !t || batch == 0 || !(lr >= 0.f))
        return dnfail(SS_ERR_INVALID_ARGUMENT, "ss_dn_train: null argument, empty batch or negative rate");
    DCK(cudaSetDevice(n->device));
    const bool update = lr > 0.f;
    DCK(cudaMemsetAsync(n->sums, 0, 2 * sizeof(double), n->stream));
    if (update) DCK(cudaMemsetAsync(n->G, 0, (size_t)kParams * sizeof(float), n->stream));
    for (uint32_t b = 0; b < batch; ++b) {
        const float *xb = x + (size_t)b * n->nvox, *tb = t + (size_t)b * n->nvox;
        enqueue_forward_act(n, xb, n->yb, n->stream);
        enqueue_backward(n, tb, n->yb, n->stream, update);
    }
    if (update) {
        n->adam_t += 1;
        const float b1 = 0.9f, b2 = 0.999f;
        const float c1 = 1.f - std::pow(b1, (float)n->adam_t), c2 = 1.f - std::pow(b2, (float)n->adam_t);
        k_dn_adam<<<(kParams + 255) / 256, 256, 0, n->stream>>>(n->P, n->G, n->M, n->S, kParams, 1.f / (float)batch,
                                                                lr, b1, b2, 1e-8f, c1, c2);
        pack_all(n, n->stream);
        n->launches += 1;
    }
    DCK(cudaGetLastError());
    double h[2];
    DCK(cudaMemcpyAsync(h, n->sums, sizeof h, cudaMemcpyDeviceToHost, n->stream));
    const int rc = check_err(n);
    if (rc != SS_OK) return rc;
    if (loss) *loss = h[0] / (double)batch;
    return SS_OK;
}

int ss_dn_gradients(ss_dn *n, const float *x, const float *t, uint32_t batch, float *grads, uint64_t count,
                    double *loss) {
    if (!n || !x || !t || !grads || batch == 0 || count != (uint64_t)kParams)
        return dnfail(SS_ERR_INVALID_ARGUMENT, "ss_dn_gradients: null argument, empty batch or count != %d", kParams);
    DCK(cudaSetDevice(n->device));
    DCK(cudaMemsetAsync(n->sums, 0, 2 * sizeof(double), n->stream));
    DCK(cudaMemsetAsync(n->G, 0, (size_t)kParams * sizeof(float), n->stream));
    for (uint32_t b = 0; b < batch; ++b) {
        const float *xb = x + (size_t)b * n->nvox, *tb = t + (size_t)b * n->nvox;
        enqueue_forward_act(n, xb, n->yb, n->stream);
        enqueue_backward(n, tb, n->yb, n->stream, true);
    }
    DCK(cudaGetLastError());
    std::vector<float> g(kParams);
    double h[2];
    DCK(cudaMemcpyAsync(g.data(), n->G, (size_t)kParams * sizeof(float), cudaMemcpyDeviceToHost, n->stream));
    DCK(cudaMemcpyAsync(h, n->sums, sizeof h, cudaMemcpyDeviceToHost, n->stream));
    const int rc = check_err(n);
    if (rc != SS_OK) return rc;
    for (int i = 0; i < kParams; ++i) grads[i] = g[i] / (float)batch;
    if (loss) *loss = h[0] / (double)batch;
    return SS_OK;
}

}  // extern "C"

extern "C" int ss_dn_sample_histogram(uint32_t nx, uint32_t ny, uint32_t np, uint64_t n, double amp, double phase,
                                      uint32_t axis, uint64_t seed, float *hist, void *stream) {
    if (!hist || nx < 1 || ny < 1 || np < 1 || n < 1 || axis > 1 || !(amp >= 0.0 && amp < 1.0) ||
        !std::isfinite(phase))
        return dnfail(SS_ERR_INVALID_ARGUMENT,
                      "ss_dn_sample_histogram: null histogram, empty grid, n = 0, axis > 1 or amp outside [0, 1)");
    cudaStream_t s = (cudaStream_t)stream;
    int dev = 0, sms = 0;
    DCK(cudaGetDevice(&dev));
    DCK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const double nbins = (double)nx * ny * np;
    const unsigned long long want = (n + 255) / 256;
    const unsigned grid = (unsigned)(want < (unsigned long long)(8 * sms) ? want : (unsigned long long)(8 * sms));
    k_dn_sample_hist<<<grid, 256, 0, s>>>((int)nx, (int)ny, (int)np, n, (float)amp, (float)phase, (int)axis, seed,
                                          (float)(nbins / (double)n), hist);
    DCK(cudaGetLastError());
    return SS_OK;
}

namespace ss {
void dn_shape(const ss_dn *n, int *nx, int *ny, int *np) {
    *nx = n->d.nx;
    *ny = n->d.ny;
    *np = n->d.np;
}
int dn_enqueue_forward(ss_dn *n, const float *x, float *y, cudaStream_t s) {
    enqueue_forward(n, x, y, s);
    return 6;
}
int dn_status(ss_dn *n, cudaStream_t s) {
    unsigned h = 0;
    DCK(cudaMemcpyAsync(&h, n->err, sizeof h, cudaMemcpyDeviceToHost, s));
    DCK(cudaStreamSynchronize(s));
    if (h) return dnfail(SS_ERR_CUDA, "denoiser: a tensor-core convolution's mbarrier wait timed out");
    return SS_OK;
}
}  // namespace ss
