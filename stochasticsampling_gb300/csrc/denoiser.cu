// denoiser.cu -- the learned histogram denoiser: a 3-D CNN (4 convolutions
// of 3x3x3 with periodic padding, 32 channels, ReLU, residual) that maps a
// low-particle-count histogram on the (x, y, phi) grid to an estimate of the
// high-count distribution before the stress / Stokes solve.
//
// Activations are BF16 in the layout [x][phi][4 chunks][y][8 channels]:
// along a line (x, phi) each 8-channel chunk is a contiguous plane of ny
// rows of 16 B, so the 128 voxels of one tile are four 2 KB blocks.  Every
// layer runs on the 5th-generation tensor cores (BF16 operands in shared
// memory, FP32 accumulators in tensor memory):
//  - k_conv32: the 32 -> 32 convolutions (and, with the weights of output
//    channel 0 alone, the 32 -> 1 output layer) as implicit GEMMs.  A tile
//    is two output rows (x, x + 1) x 128 y at one phi; a CTA walks along phi
//    through its runs of tiles; each input position (the 4 lines x - 1 ..
//    x + 2 at one phi, with one halo row at either end, periodic in y) lands
//    in a ring of position buffers by bulk copies from a producer warp, and
//    the taps are descriptor offsets into those lines (the y shift is a
//    16-byte row offset).  A position feeds the output tiles phi - 1, phi and
//    phi + 1, so each (row, dx, dy, K half) is one MMA of M = 128, N = 96
//    (K = 16) with the three dphi taps' weights stacked along N.  The MMA
//    warp runs its loop warp-uniformly with one elected lane issuing into
//    two rings of 8 accumulators; eight epilogue warps drain finished
//    accumulators with tcgen05.ld (one voxel's 32 channels per thread) and
//    apply bias and ReLU, the ReLU derivative of a reference tensor (the
//    backward pass) or the residual (the output layer).
//  - k_dn_in_tc: the 1 -> 32 input layer, one small GEMM per tile with the
//    27 taps as K; k_dn_wgrad_tc / k_dn_wgrad1_tc: the weight gradients, GEMMs
//    over the voxels with the accumulators resident in tensor memory and
//    fixed-order sums over the CTAs.
// The same GEMM, on dy with mirrored weights, is the output layer's backward.
// The CUDA cores keep the layout transposes, the loss, Adam and the weight
// packing.
//
// Shared-memory operand layouts (no swizzle).  A line (K-major): for each of
// its 4 K chunks (8 channels, 16 bytes) the rows at a 16-byte stride, so row
// groups are 128 B apart (stride offset) and K chunks 2176 B (leading
// offset).  Weights (K-major): per tap 32 rows x 4 chunks in 8 x 16 B core
// matrices, leading offset 128 B, stride offset 512 B.  Every wait is
// bounded: on a timeout a kernel records an error, waits for its own copies
// and MMAs, frees its tensor memory and returns.
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
// A line buffer: 4 K chunks (8 channels, 16 B per row) of 136 rows each.
// Rows 8 .. 135 of a chunk hold y0 .. y0 + 127 (one 2 KB bulk copy), row 7
// the halo y0 - 1; the halo y0 + 128 sits in row 136, which is row 0 of the
// next chunk (rows 0 .. 6 of a chunk are never read), and for the last
// chunk in the 128 bytes past it.
constexpr int kChunkRows = 136;
constexpr int kChunkBytes = kChunkRows * 16;       // 2176 B: the A operand's leading offset
constexpr int kBodyOff = 8 * 16;                   // byte offset of row y0 in a chunk
constexpr int kLineBytes = 4 * kChunkBytes + 128;  // 8832 B
constexpr int kBodyBytes = kTileM * 16;            // one chunk of 128 rows
constexpr int kAccStages = 8;                      // accumulators of 32 columns in tensor memory (a ring)
constexpr int kWgThreads = 192;  // the weight gradient: warp 0 loads, warps 1-2 issue MMAs, warps 2-5 write the sums
constexpr int kBarBytes = 512;
// The convolution's shape by the number of output rows (along x) a tile
// covers: ROWS rows take ROWS + 2 input lines per position (a position
// buffer), ROWS rings of kAccStages accumulators in tensor memory and 4
// epilogue warps per row; as many position buffers as fit beside the
// weights (at most 6).  Two rows per tile read 2 lines per output row
// instead of 3.
template <int ROWS>
struct ConvShape {
    static constexpr int kLines = ROWS + 2;
    static constexpr int kPosBytes = kLines * kLineBytes;
    static constexpr int kFree = 227 * 1024 - 1024 - kBAll - kBarBytes - 16;  // + alignment slack
    static constexpr int kSlots = kFree / kPosBytes < 6 ? kFree / kPosBytes : 6;
    static constexpr int kThreads = 64 + 128 * ROWS;
    static constexpr int kTmemCols = 32 * kAccStages * ROWS;
    static constexpr int kSmem = 1024 + kBAll + kSlots * kPosBytes + kBarBytes + 16;
    static_assert(kSlots >= 3, "fewer than 3 position buffers fit in shared memory");
    static_assert(kTmemCols <= 512, "the accumulator rings exceed the tensor memory");
};
constexpr int kConvRows = 2;  // output rows per tile of the 32 -> 32 convolution
static_assert(8 * (2 * 6 + 2 * kAccStages + 2) <= kBarBytes, "mbarriers do not fit");
static_assert(kBAll % 16 == 0 && kLineBytes % 16 == 0 && kChunkBytes % 16 == 0, "bulk copies need 16-B alignment");
constexpr uint32_t kWaitLimit = 1u << 22;    // mbarrier polls before giving up
constexpr unsigned kErrTimeout = 1u;

struct Dims {
    int nx, ny, np;
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// i in [-n, 2n) wrapped into [0, n)
__device__ __forceinline__ int wrap_idx(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

// ---- PTX wrappers ------------------------------------------------------
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
// the same, giving up early once another role of the CTA has failed
__device__ __forceinline__ bool mbar_wait_or_fail(uint32_t addr, uint32_t parity, const volatile int *fail) {
    for (uint32_t i = 0; i < kWaitLimit; ++i) {
        if (mbar_try_wait(addr, parity)) return true;
        if ((i & 255u) == 255u && *fail) return false;
    }
    return false;
}
// a wait of a role off the MMA thread's critical path: polls with a short pause so
// that it takes few issue slots from the warps it shares a scheduler with
__device__ __forceinline__ bool mbar_wait_polite(uint32_t addr, uint32_t parity, const volatile int *fail) {
    for (uint32_t i = 0; i < kWaitLimit; ++i) {
        if (mbar_try_wait(addr, parity)) return true;
        if ((i & 15u) == 15u && *fail) return false;
        __nanosleep(64);
    }
    return false;
}
// a long wait (the whole kernel): polls with a 256 ns pause, giving up after ~1 s or
// once another role of the CTA has failed
__device__ __forceinline__ bool mbar_wait_long(uint32_t addr, uint32_t parity, const volatile int *fail) {
    for (uint32_t i = 0; i < kWaitLimit; ++i) {
        if (mbar_try_wait(addr, parity)) return true;
        if (*fail) return false;
        __nanosleep(256);
    }
    return false;
}
__device__ __forceinline__ void mbar_arrive(uint32_t addr) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(addr) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t addr, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(addr), "r"(bytes) : "memory");
}
__device__ __forceinline__ void st_shared16(uint32_t addr, uint4 v) {
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};\n" ::"r"(addr), "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w)
                 : "memory");
}
// bytes (a multiple of 16) from global src to shared dst, both 16-byte aligned,
// completing as transactions on mbar
__device__ __forceinline__ void bulk_load(uint32_t dst, const void *src, uint32_t bytes, uint32_t mbar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(mbar)
                 : "memory");
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
// D[tmem] (+)= A[smem] * B[smem]^T, kind::f16 (BF16 operands, FP32 accumulator),
// issued by the calling thread
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
// mbarrier arrival once the calling thread's MMAs issued so far have completed
__device__ __forceinline__ void mma_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar)
                 : "memory");
}
// the same two from a whole converged warp: one elected lane (the same one
// every time, so that its commits cover its MMAs) issues, and the warp's
// descriptor arithmetic stays warp-uniform
__device__ __forceinline__ void mma_bf16_warp(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                              uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred e, p;\n .reg .b32 l;\n elect.sync l|e, 0xffffffff;\n setp.ne.b32 p, %4, 0;\n"
        " @e tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void mma_commit_warp(uint32_t mbar) {
    asm volatile(
        "{\n .reg .pred e;\n .reg .b32 l;\n elect.sync l|e, 0xffffffff;\n"
        " @e tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n}\n" ::"r"(mbar)
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

// instruction descriptor: D FP32, A and B BF16, both K-major, M = 128 (N in bits 17-22, in units of 8)
constexpr uint32_t kIdescM128 = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kTileM >> 4) << 24);
// Shared-memory matrix descriptors (no swizzle): start address >> 4 in bits
// 0-13, leading offset >> 4 in bits 16-29, stride offset >> 4 in bits 32-45,
// version 1 in bit 46.  The convolution's operands are K-major: a line's K
// chunks 2176 B apart and its 8-row groups 128 B apart; the weights' K chunks
// 128 B apart and their 8-row groups 512 B apart.
constexpr uint64_t kADesc = ((uint64_t)(kChunkBytes >> 4) << 16) | ((uint64_t)(128 >> 4) << 32) | (1ull << 46);
constexpr uint64_t kBDesc = ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(512 >> 4) << 32) | (1ull << 46);
// start-address offsets (>> 4) of the (dx, dy, K half) product (indices 0-2, 0-2, 0-1) within a
// position buffer and within the packed weights
__host__ __device__ constexpr uint64_t a_off(int dx, int dy, int kk) {
    return (uint64_t)((dx * kLineBytes + kk * 2 * kChunkBytes + kBodyOff + (dy - 1) * 16) >> 4);
}
__host__ __device__ constexpr uint64_t b_off(int dx, int dy, int kk) {
    return (uint64_t)(((dx * 9 + dy * 3) * kBTap + kk * 256) >> 4);
}
// one piece of a position's MMAs: the accumulator columns of consecutive tiles
struct Piece {
    uint32_t col;    // tensor-memory address of the first tile's accumulator
    uint32_t idesc;  // instruction descriptor (N = 32 x tiles)
    uint64_t boff;   // offset (>> 4) of the first tile's weight block within a triple
    uint32_t acc;    // accumulate (0: the first product of the piece's tiles)
};
// the 17 (dx, dy, K half) products after the first, NP pieces each, for
// each of ROWS output rows (row r reads the position's lines r .. r + 2 and
// accumulates into ring r, kAccStages * 32 columns further on)
template <int NP, int ROWS>
__device__ __forceinline__ void issue_rest(uint64_t adesc0, uint64_t bdesc0, const Piece *pp) {
#pragma unroll
    for (int t = 1; t < 18; ++t) {
        const int dx = t / 6, dy = (t / 2) % 3, kk = t % 2;
        const uint64_t a = adesc0 + a_off(dx, dy, kk), b = bdesc0 + b_off(dx, dy, kk);
#pragma unroll
        for (int k = 0; k < NP; ++k)
#pragma unroll
            for (int r = 0; r < ROWS; ++r)
                mma_bf16_warp(pp[k].col + (uint32_t)(32 * kAccStages * r), a + (uint64_t)r * (kLineBytes >> 4),
                              b + pp[k].boff, pp[k].idesc, 1u);
    }
}

// byte offset of element (row, k) of a K-major operand block in the core-matrix layout
__host__ __device__ __forceinline__ int core_offset(int row, int k) {
    return (row >> 3) * 512 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2;
}

// MODE 0: bias + ReLU -> BF16; MODE 1: bias -> FP32; MODE 2: times ReLU'(ref) -> BF16;
// MODE 3: the 32 -> 1 output layer (weights of output channel 0, the other 31
// zero): res + channel 0 + bias -> FP32 in the layout [x][phi][y].
// ny a multiple of 128.  Output tiles (ROWS rows x .. x + ROWS - 1, y
// segment, phi) in the order phi fastest; CTA b takes the contiguous range
// [b T / grid, (b + 1) T / grid) of the T tiles and walks it in runs of
// consecutive phi at one (x, y segment).  A run of L tiles streams its L + 2
// input positions along phi; a position holds the ROWS + 2 lines x - 1 ..
// x + ROWS (periodic), and for each output row r the 3 lines r .. r + 2
// (dx = -1, 0, 1) of input position p feed the output tiles p + 1, p and
// p - 1 (dphi = -1, 0, +1), so one MMA of N = 96 covers all three with the
// weights of the three dphi taps stacked along N (the packed weights keep
// each (dx, dy) triple in the order dphi = +1, 0, -1): 18 MMAs per row and
// input position instead of 54 of N = 32.  The accumulators of
// consecutive tiles are consecutive 32-column stages of a ring in tensor
// memory; an MMA is split where the ring wraps, and where a tile takes its
// first product (accumulate off).  The tensor core takes an N = 96 MMA every
// 56 cycles, so the issuing thread's loop is kept to a few instructions per
// MMA: 64-bit descriptors plus compile-time offsets, and a branch-free path
// for positions whose tiles lie in one piece of the ring.  Roles,
// synchronised through mbarriers with bounded waits:
//  - warp 0 streams positions into a ring of position buffers with bulk
//    copies (cp.async.bulk), 4 (ROWS + 2) lanes at once (one bulk copy
//    costs its issuing thread some 80 cycles): per line its 4 chunk bodies
//    (2 KB each, contiguous in the activation layout) and its 8 halo pieces
//    (16 B, periodic in y) straight into rows 7 and 136; full[slot]
//    completes when the position's (ROWS + 2) x 8,320 bytes are in;
//  - warp 1 (one thread) waits for the position and, when a tile starts,
//    for its accumulator stage to be free; issues the MMAs of every row
//    (row r into its own ring); returns the position's buffer to the
//    producer (empty[slot]) and commits the tile that the position
//    completed to acc_full[stage];
//  - warps 2 + 4 r .. 5 + 4 r wait for acc_full, read row r's accumulator
//    (warp w the tensor-memory lanes 32 (w mod 4) ..), release it to
//    acc_empty and write the outputs, while the tensor core already runs
//    the next positions.
template <int MODE, int ROWS>
__global__ void __launch_bounds__(ConvShape<ROWS>::kThreads, 1) k_conv32(const __nv_bfloat16 *__restrict__ X,
                                                                         const uint8_t *__restrict__ Wpacked,
                                                                         const float *__restrict__ bias,
                                                                         const __nv_bfloat16 *__restrict__ ref,
                                                                         const float *__restrict__ res,
                                                                         void *__restrict__ Y, Dims d,
                                                                         unsigned *__restrict__ err) {
    using CS = ConvShape<ROWS>;
    constexpr int kSlots = CS::kSlots;
    extern __shared__ uint8_t smem_raw[];
    const uint32_t raw = smem_u32(smem_raw);
    const uint32_t sB0 = (raw + 1023u) & ~1023u;
    uint8_t *const sB = smem_raw + (sB0 - raw);
    const uint32_t sL0 = sB0 + kBAll;
    const uint32_t bar0 = sL0 + kSlots * CS::kPosBytes;
    auto full_bar = [&](uint32_t s) { return bar0 + 8u * s; };
    auto empty_bar = [&](uint32_t s) { return bar0 + 8u * (kSlots + s); };
    auto accf_bar = [&](uint32_t a) { return bar0 + 8u * (2 * kSlots + a); };
    auto acce_bar = [&](uint32_t a) { return bar0 + 8u * (2 * kSlots + kAccStages + a); };
    const uint32_t fin_bar = bar0 + 8u * (2 * kSlots + 2 * kAccStages);
    const uint32_t w_bar = fin_bar + 8u;  // the weights have landed
    uint32_t *tslot = reinterpret_cast<uint32_t *>(sB + kBAll + kSlots * CS::kPosBytes + kBarBytes);
    volatile int *sfail = reinterpret_cast<volatile int *>(tslot + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    if (tid == 0) {
        for (int s = 0; s < kSlots; ++s) {
            mbar_init(full_bar(s), 1);  // the expect_tx arrival (+ the transactions)
            mbar_init(empty_bar(s), 1);
        }
        for (int a = 0; a < kAccStages; ++a) {
            mbar_init(accf_bar(a), 1);
            mbar_init(acce_bar(a), 4 * ROWS);  // one arrival per epilogue warp
        }
        mbar_init(fin_bar, 1);
        mbar_init(w_bar, 1);
        *sfail = 0;
        fence_mbar_init();
    }
    if (warp == 1) tmem_alloc(smem_u32(tslot), CS::kTmemCols);
    fence_proxy_async();
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    const uint32_t tmem = *tslot;

    const int nseg = d.ny / kTileM;
    const int T = ((d.nx + ROWS - 1) / ROWS) * nseg * d.np;
    const int t0 = (int)((long long)blockIdx.x * T / gridDim.x);
    const int t1 = (int)((long long)(blockIdx.x + 1) * T / gridDim.x);
    // tile t -> (first row x, y0, p)
    auto decode = [&](int t, int &x, int &y0, int &p) {
        p = t % d.np;
        y0 = ((t / d.np) % nseg) * kTileM;
        x = (t / (d.np * nseg)) * ROWS;
    };
    auto wrapi = [](int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); };

    if (warp == 0) {
        // ---- producer: the ROWS + 2 lines of every input position of every run; lane 4 l + c
        // copies chunk c of line l (x - 1 + l, periodic): its body and its two halo rows ----
        uint32_t pos = 0;  // the CTA's count of input positions
        bool ok = true;
        // the packed weights (54 KB, one bulk copy), landing while the first positions stream in
        if (lane == 0) {
            mbar_expect_tx(w_bar, (uint32_t)kBAll);
            bulk_load(sB0, Wpacked, (uint32_t)kBAll, w_bar);
        }
        __syncwarp();
        for (int r0 = t0; r0 < t1 && ok;) {
            int x, y0, pa;
            decode(r0, x, y0, pa);
            const int L = min(t1 - r0, d.np - pa);
            const int ytop = wrapi(y0 - 1, d.ny), ybot = wrapi(y0 + kTileM, d.ny);
            for (int j = 0; j < L + 2; ++j, ++pos) {
                const uint32_t slot = pos % kSlots;
                if (pos >= (uint32_t)kSlots)
                    ok = mbar_wait_polite(empty_bar(slot), ((pos / kSlots) - 1u) & 1u, sfail);
                ok = __all_sync(0xffffffffu, ok);
                if (!ok) break;
                const int pin = wrapi(pa - 1 + j, d.np);
                if (lane == 0) mbar_expect_tx(full_bar(slot), (uint32_t)CS::kLines * 4u * (kBodyBytes + 32u));
                __syncwarp();
                if (lane < 4 * CS::kLines) {
                    const int dx = lane >> 2, c = lane & 3;
                    // line x - 1 + dx, periodic (x - 1 + dx lies in [-1, nx + ROWS])
                    const int xl = (x + dx - 1 + 2 * d.nx) % d.nx;
                    // chunk plane c of the line: ny rows of 16 B from X + (line 4 + c) ny 8
                    const __nv_bfloat16 *pc = X + ((size_t)(xl * d.np + pin) * 4 + c) * d.ny * 8;
                    const uint32_t dc = sL0 + slot * (uint32_t)CS::kPosBytes + (uint32_t)(dx * kLineBytes + c * kChunkBytes + kBodyOff);
                    bulk_load(dc, pc + (size_t)y0 * 8, kBodyBytes, full_bar(slot));
                    bulk_load(dc - 16, pc + (size_t)ytop * 8, 16, full_bar(slot));
                    bulk_load(dc + kBodyBytes, pc + (size_t)ybot * 8, 16, full_bar(slot));
                }
                __syncwarp();
            }
            r0 += L;
        }
        if (!ok && lane == 0) *sfail = 1;
        // every load issued lands before the CTA may exit
        if (lane == 0) {
            for (uint32_t q = pos > (uint32_t)kSlots ? pos - kSlots : 0u; q < pos; ++q)
                if (!mbar_wait(full_bar(q % kSlots), (q / kSlots) & 1u)) *sfail = 1;
            if (!mbar_wait(w_bar, 0)) *sfail = 1;
        }
    } else if (warp == 1) {
        // ---- MMA issuer: the whole warp runs the loop (warp-uniform), one elected lane issues ----
        {
            uint32_t pos = 0;
            int ibase = 0;  // the CTA's count of tiles before this run (accumulator stage = count mod kAccStages)
            bool ok = true;
            const uint64_t bdesc0 = kBDesc | (uint64_t)((sB0 >> 4) & 0x3FFFu);
            ok = __all_sync(0xffffffffu, mbar_wait_or_fail(w_bar, 0, sfail));
            for (int r0 = t0; r0 < t1 && ok;) {
                int x, y0, pa;
                decode(r0, x, y0, pa);
                const int L = min(t1 - r0, d.np - pa);
                for (int j = 0; j < L + 2; ++j, ++pos) {
                    const uint32_t slot = pos % kSlots;
                    ok = __all_sync(0xffffffffu, mbar_wait_or_fail(full_bar(slot), (pos / kSlots) & 1u, sfail));
                    // tile j starts at this position: its stage's previous tile has left it
                    const int inew = ibase + j;
                    if (ok && j < L && inew >= kAccStages)
                        ok = __all_sync(0xffffffffu, mbar_wait_or_fail(acce_bar(inew % kAccStages),
                                                                       ((inew / kAccStages) - 1) & 1, sfail));
                    if (!ok) break;
                    tc_after_sync();
                    // plan: tiles lo..hi take this position's products; tile k's block in the weight
                    // triple is k - j + 2 (dphi = +1, 0, -1); pieces split where the stage ring wraps
                    const int lo = j - 2 > 0 ? j - 2 : 0, hi = j < L - 1 ? j : L - 1;
                    Piece pp[2], pq[3];
                    int np_ = 0, nq = 0;
                    auto split = [&](int klo, int khi, Piece *pc, int &cnt) {
                        if (klo > khi) return;
                        const int s0 = (ibase + klo) & (kAccStages - 1), tot = khi - klo + 1;
                        const int n1 = tot < kAccStages - s0 ? tot : kAccStages - s0;
                        pc[cnt++] = Piece{tmem + (uint32_t)(32 * s0), kIdescM128 | ((uint32_t)(4 * n1) << 17),
                                          (uint64_t)((klo - j + 2) * (kBTap >> 4)), 1u};
                        if (n1 < tot)
                            pc[cnt++] = Piece{tmem, kIdescM128 | ((uint32_t)(4 * (tot - n1)) << 17),
                                              (uint64_t)((klo + n1 - j + 2) * (kBTap >> 4)), 1u};
                    };
                    split(lo, hi, pp, np_);
                    if (j < L) {
                        pq[0] = Piece{tmem + (uint32_t)(32 * ((ibase + j) & (kAccStages - 1))), kIdescM128 | (4u << 17),
                                      (uint64_t)(2 * (kBTap >> 4)), 0u};  // tile j's first product
                        nq = 1;
                        split(lo, j - 1, pq, nq);
                    } else {
                        pq[0] = pp[0];
                        pq[1] = pp[1];
                        nq = np_;
                    }
                    const uint64_t adesc0 =
                        kADesc | (uint64_t)(((sL0 + slot * (uint32_t)CS::kPosBytes) >> 4) & 0x3FFFu);
                    // the first (dx, dy, K half) product with the first-product plan, then the 17 others
                    for (int k = 0; k < nq; ++k)
#pragma unroll
                        for (int r = 0; r < ROWS; ++r)
                            mma_bf16_warp(pq[k].col + (uint32_t)(32 * kAccStages * r),
                                          adesc0 + a_off(0, 0, 0) + (uint64_t)r * (kLineBytes >> 4),
                                          bdesc0 + b_off(0, 0, 0) + pq[k].boff, pq[k].idesc, pq[k].acc);
                    if (np_ == 1) issue_rest<1, ROWS>(adesc0, bdesc0, pp);
                    else issue_rest<2, ROWS>(adesc0, bdesc0, pp);
                    mma_commit_warp(empty_bar(slot));
                    if (j >= 2) mma_commit_warp(accf_bar((ibase + j - 2) % kAccStages));  // tile j - 2 is complete
                }
                ibase += L;
                r0 += L;
            }
            if (!ok) *sfail = 1;
            // the MMAs issued complete before the tensor memory is freed
            mma_commit_warp(fin_bar);
            if (!mbar_wait(fin_bar, 0)) *sfail = 1;
        }
        __syncwarp();
    } else if (warp >= 2) {
        // ---- epilogue: warps 2 + 4 g .. 5 + 4 g drain row g ----
        const int q = warp & 3;  // tensor-memory lanes 32 q .. 32 q + 31
        const int g = (warp - 2) >> 2;
        int i = 0;
        for (int t = t0; t < t1; ++t, ++i) {
            const int a = i % kAccStages;
            // tcgen05.ld wants the whole warp: the lanes leave together
            if (!__all_sync(0xffffffffu, mbar_wait_polite(accf_bar(a), (i / kAccStages) & 1, sfail))) {
                *sfail = 1;
                break;
            }
            tc_after_sync();
            uint32_t r[32];
            tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(32 * kAccStages * g + 32 * a), r);
            tc_before_sync();
            __syncwarp();
            if (lane == 0) mbar_arrive(acce_bar(a));
            int x, y0, p;
            decode(t, x, y0, p);
            x += g;
            if (x >= d.nx) continue;  // the second row of the last tile of an odd nx
            // this thread's voxel: row y of line x np + p; chunk plane c at (line 4 + c) ny
            const size_t line = (size_t)x * d.np + p, y = (size_t)(y0 + q * 32 + lane);
            auto at = [&](int c) { return ((line * 4 + c) * d.ny + y) * 8; };
            if (MODE == 3) {
                const size_t v = line * d.ny + y;
                reinterpret_cast<float *>(Y)[v] = res[v] + __uint_as_float(r[0]) + bias[0];
            } else if (MODE == 1) {
                float *out = reinterpret_cast<float *>(Y);
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    float4 *o = reinterpret_cast<float4 *>(out + at(c));
                    o[0] = make_float4(__uint_as_float(r[8 * c]) + bias[8 * c], __uint_as_float(r[8 * c + 1]) + bias[8 * c + 1],
                                       __uint_as_float(r[8 * c + 2]) + bias[8 * c + 2],
                                       __uint_as_float(r[8 * c + 3]) + bias[8 * c + 3]);
                    o[1] = make_float4(__uint_as_float(r[8 * c + 4]) + bias[8 * c + 4],
                                       __uint_as_float(r[8 * c + 5]) + bias[8 * c + 5],
                                       __uint_as_float(r[8 * c + 6]) + bias[8 * c + 6],
                                       __uint_as_float(r[8 * c + 7]) + bias[8 * c + 7]);
                }
            } else {
                uint32_t packed[16];
                uint32_t mask[16];
                if (MODE == 2) {
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        const uint4 u = *reinterpret_cast<const uint4 *>(ref + at(c));
                        mask[4 * c] = u.x;
                        mask[4 * c + 1] = u.y;
                        mask[4 * c + 2] = u.z;
                        mask[4 * c + 3] = u.w;
                    }
                }
#pragma unroll
                for (int c = 0; c < 16; ++c) {
                    float a0 = __uint_as_float(r[2 * c]), b0 = __uint_as_float(r[2 * c + 1]);
                    if (MODE == 0) {
                        a0 = fmaxf(a0 + bias[2 * c], 0.f);
                        b0 = fmaxf(b0 + bias[2 * c + 1], 0.f);
                    } else {
                        const __nv_bfloat162 m = *reinterpret_cast<const __nv_bfloat162 *>(&mask[c]);
                        a0 = __low2float(m) > 0.f ? a0 : 0.f;
                        b0 = __high2float(m) > 0.f ? b0 : 0.f;
                    }
                    __nv_bfloat162 h = __floats2bfloat162_rn(a0, b0);
                    packed[c] = *reinterpret_cast<uint32_t *>(&h);
                }
                __nv_bfloat16 *out = reinterpret_cast<__nv_bfloat16 *>(Y);
#pragma unroll
                for (int c = 0; c < 4; ++c)
                    *reinterpret_cast<uint4 *>(out + at(c)) =
                        make_uint4(packed[4 * c], packed[4 * c + 1], packed[4 * c + 2], packed[4 * c + 3]);
            }
        }
    }
    __syncthreads();
    if (*sfail && tid == 0) atomicOr(err, kErrTimeout);
    tc_after_sync();
    if (warp == 1) tmem_dealloc(tmem, CS::kTmemCols);
}

// Weight gradient of a 32 -> 32 layer on the tensor cores:
//   dW[tap][co][ci] = sum_v dZ[v][co] A[nbr(v, tap)][ci],   db[co] = sum_v dZ[v][co].
// A GEMM over voxels: D[(4 lines x 32 ci) = 128][32 co] += X_rows[128][16 voxels]
// dZ[32][16 voxels]^T, both operands MN-major in shared memory (no swizzle):
// a core matrix is 8 voxels x 8 channels, one 16-byte row per voxel, which is
// how a line buffer already holds its chunks, so the dy shift is again a
// 16-byte row offset and the 4 lines of one MMA are 4 consecutive line slots
// (M-group stride = the chunk stride, 2176 B, with line slots exactly 4
// chunks long).  Per tile (x, y segment, phi) the 9 lines (dx, dphi) and the
// tile's dZ are bulk-copied into one of two buffers; the 27 taps are 3 MMAs
// of M = 128 per (dy, 16-voxel step): lines 0-3, 4-7 and 8 plus a line of
// ones (its rows give db) and two slots whose rows are discarded.  9
// accumulators of 32 columns persist in tensor memory over the CTA's tiles;
// at the end the CTA writes its partial sums, and k_dn_wgrad_reduce adds
// the CTAs' partials in a fixed order.
constexpr int kWgSlotBytes = 4 * kChunkBytes;        // 8704 B: lines back to back at the M-group stride
constexpr int kWgBufSlots = 10;                      // 9 lines + the ones line
constexpr int kWgSlots = 2 * kWgBufSlots + 2;        // two buffers + 2 slots the last group's discarded rows read
constexpr int kWgDzBytes = 4 * kBodyBytes;           // a tile's dZ: 4 chunks of 128 rows
constexpr int kWgPartial = kTaps * kC * kC + kC;     // floats per CTA: dW then db
constexpr int kSmemWg = 1024 + 2 * kWgDzBytes + kWgSlots * kWgSlotBytes + 128 + 64;
static_assert(kSmemWg <= 227 * 1024, "the weight gradient's shared memory exceeds a CTA's limit");
// M = 128, N = 32, A and B MN-major (bits 15, 16)
constexpr uint32_t kIdescWg = kIdescM128 | (4u << 17) | (1u << 15) | (1u << 16);

__global__ void __launch_bounds__(kWgThreads, 1) k_dn_wgrad_tc(const __nv_bfloat16 *__restrict__ dZ,
                                                                 const __nv_bfloat16 *__restrict__ X,
                                                                 float *__restrict__ partial, Dims d,
                                                                 unsigned *__restrict__ err) {
    extern __shared__ uint8_t smem_raw[];
    const uint32_t raw = smem_u32(smem_raw);
    const uint32_t sZ0 = (raw + 1023u) & ~1023u;  // dZ buffers
    uint8_t *const sZ = smem_raw + (sZ0 - raw);
    const uint32_t sS0 = sZ0 + 2 * kWgDzBytes;    // line slots
    const uint32_t bar0 = sS0 + kWgSlots * kWgSlotBytes + 128;
    auto full_bar = [&](uint32_t b) { return bar0 + 8u * b; };
    auto empty_bar = [&](uint32_t b) { return bar0 + 16u + 8u * b; };
    const uint32_t fin_bar = bar0 + 32u;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(sZ + (bar0 + 40u - sZ0));
    volatile int *sfail = reinterpret_cast<volatile int *>(tslot + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    // the ones lines (rows y0 .. y0 + 127 of every chunk of slot 9 of each buffer)
    for (int i = tid; i < 2 * 4 * kTileM; i += kWgThreads) {
        const int b = i / (4 * kTileM), c = (i / kTileM) % 4, r = i % kTileM;
        const uint32_t one2 = 0x3F803F80u;  // two BF16 1.0
        st_shared16(sS0 + (uint32_t)((b * kWgBufSlots + 9) * kWgSlotBytes + c * kChunkBytes + kBodyOff + r * 16),
                    make_uint4(one2, one2, one2, one2));
    }
    if (tid == 0) {
        for (int b = 0; b < 2; ++b) {
            mbar_init(full_bar(b), 1);
            mbar_init(empty_bar(b), 2);  // both issuers' commits
        }
        mbar_init(fin_bar, 2);
        *sfail = 0;
        fence_mbar_init();
    }
    if (warp == 1) tmem_alloc(smem_u32(tslot), 512);
    fence_proxy_async();
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    const uint32_t tmem = *tslot;

    const int nseg = d.ny / kTileM;
    const int T = d.nx * nseg * d.np;
    const int t0 = (int)((long long)blockIdx.x * T / gridDim.x);
    const int t1 = (int)((long long)(blockIdx.x + 1) * T / gridDim.x);
    auto wrapi = [](int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); };

    if (warp == 0) {
        // ---- producer: per tile 9 lines (4 chunks: body + 2 halo rows each) and the tile's dZ;
        // the 36 (line, chunk) pairs go to the 32 lanes in two passes ----
        bool ok = true;
        int i = 0;
        for (int t = t0; t < t1; ++t, ++i) {
            const int b = i & 1;
            if (i >= 2) ok = mbar_wait_or_fail(empty_bar(b), ((i >> 1) - 1) & 1, sfail);
            ok = __all_sync(0xffffffffu, ok);
            if (!ok) break;
            const int p = t % d.np, y0 = ((t / d.np) % nseg) * kTileM, x = t / (d.np * nseg);
            const int ytop = wrapi(y0 - 1, d.ny), ybot = wrapi(y0 + kTileM, d.ny);
            if (lane == 0) mbar_expect_tx(full_bar(b), 9u * 4u * (kBodyBytes + 32u) + (uint32_t)kWgDzBytes);
            __syncwarp();
            for (int e = lane; e < 36; e += 32) {
                const int l = e >> 2, c = e & 3, dx = l / 3 - 1, dp = l % 3 - 1;
                const __nv_bfloat16 *pc =
                    X + ((size_t)(wrapi(x + dx, d.nx) * d.np + wrapi(p + dp, d.np)) * 4 + c) * d.ny * 8;
                const uint32_t dc = sS0 + (uint32_t)((b * kWgBufSlots + l) * kWgSlotBytes + c * kChunkBytes + kBodyOff);
                bulk_load(dc, pc + (size_t)y0 * 8, kBodyBytes, full_bar(b));
                bulk_load(dc - 16, pc + (size_t)ytop * 8, 16, full_bar(b));
                bulk_load(dc + kBodyBytes, pc + (size_t)ybot * 8, 16, full_bar(b));
            }
            if (lane >= 4 && lane < 8) {
                const int c = lane - 4;
                bulk_load(sZ0 + (uint32_t)(b * kWgDzBytes + c * kBodyBytes),
                          dZ + (((size_t)(x * d.np + p) * 4 + c) * d.ny + y0) * 8, kBodyBytes, full_bar(b));
            }
            __syncwarp();
        }
        if (!ok && lane == 0) *sfail = 1;
        // the loads issued land before the CTA may exit
        if (lane == 0)
            for (int k = i > 2 ? i - 2 : 0; k < i; ++k)
                if (!mbar_wait(full_bar(k & 1), (k >> 1) & 1)) *sfail = 1;
    } else if ((warp == 1 || warp == 2) && lane == 0) {
        // ---- two MMA issuers: warp 1 the accumulators (dy, group) 0-4, warp 2 the accumulators 5-8;
        // disjoint, so each accumulator's products keep one order ----
        constexpr uint64_t kAWg = ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(kChunkBytes >> 4) << 32) | (1ull << 46);
        constexpr uint64_t kBWg = ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(kBodyBytes >> 4) << 32) | (1ull << 46);
        bool ok = true;
        int i = 0;
        for (int t = t0; t < t1; ++t, ++i) {
            const int b = i & 1;
            if (!mbar_wait_or_fail(full_bar(b), (i >> 1) & 1, sfail)) {
                ok = false;
                break;
            }
            tc_after_sync();
            const uint64_t a0 = kAWg | (uint64_t)(((sS0 + (uint32_t)(b * kWgBufSlots * kWgSlotBytes)) >> 4) & 0x3FFFu);
            const uint64_t z0 = kBWg | (uint64_t)(((sZ0 + (uint32_t)(b * kWgDzBytes)) >> 4) & 0x3FFFu);
            const uint32_t acc0 = i > 0 ? 1u : 0u;
#pragma unroll
            for (int kk = 0; kk < kTileM / 16; ++kk) {
                const uint32_t acc = kk > 0 ? 1u : acc0;
                const uint64_t bd = z0 + (uint64_t)(kk * 256 >> 4);
                if (warp == 1) {
#pragma unroll
                    for (int a = 0; a < 5; ++a) {
                        const int dy = a / 3, g = a % 3;
                        mma_bf16(tmem + (uint32_t)(32 * a),
                                 a0 + (uint64_t)((g * 4 * kWgSlotBytes + kBodyOff + (16 * kk + dy - 1) * 16) >> 4), bd,
                                 kIdescWg, acc);
                    }
                } else {
#pragma unroll
                    for (int a = 5; a < 9; ++a) {
                        const int dy = a / 3, g = a % 3;
                        mma_bf16(tmem + (uint32_t)(32 * a),
                                 a0 + (uint64_t)((g * 4 * kWgSlotBytes + kBodyOff + (16 * kk + dy - 1) * 16) >> 4), bd,
                                 kIdescWg, acc);
                    }
                }
            }
            mma_commit(empty_bar(b));
        }
        if (!ok) *sfail = 1;
        mma_commit(fin_bar);
    }
    // ---- every thread: the accumulators leave once the MMAs are done ----
    // (the issuers wait without the failure shortcut: their MMAs finish before the dealloc)
    bool done = (warp == 1 || warp == 2) && lane == 0 ? mbar_wait(fin_bar, 0) : mbar_wait_long(fin_bar, 0, sfail);
    done = __all_sync(0xffffffffu, done);  // tcgen05.ld wants the whole warp
    if (warp >= 2 && done && t1 > t0) {
        const int q = warp & 3;  // tensor-memory lanes 32 q ..: rows (line 4 g + q, ci = lane)
        tc_after_sync();
        float *out = partial + (size_t)blockIdx.x * kWgPartial;
#pragma unroll 1
        for (int a = 0; a < 9; ++a) {
            const int dy = a / 3, g = a % 3, l = 4 * g + q;
            uint32_t r[32];
            tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(32 * a), r);
            if (l < 9) {
                const int tap = (l / 3) * 9 + dy * 3 + (l % 3);
#pragma unroll
                for (int co = 0; co < kC; ++co) out[(tap * kC + co) * kC + lane] = __uint_as_float(r[co]);
            } else if (l == 9 && dy == 1 && lane == 0) {
#pragma unroll
                for (int co = 0; co < kC; ++co) out[kTaps * kC * kC + co] = __uint_as_float(r[co]);
            }
        }
    } else if (warp >= 2 && t1 <= t0) {
        float *out = partial + (size_t)blockIdx.x * kWgPartial;
        for (int e = tid - 64; e < kWgPartial; e += kWgThreads - 64) out[e] = 0.f;
    }
    if (!done) *sfail = 1;
    tc_before_sync();
    __syncthreads();
    if (*sfail && tid == 0) atomicOr(err, kErrTimeout);
    tc_after_sync();
    if (warp == 1) tmem_dealloc(tmem, 512);
}

// Weight gradients of the 1-channel layers on the tensor cores.  Per tile of
// 128 voxels (x, phi, y0 .. y0 + 127) one GEMM over the voxels,
//   D[r][c] += sum_v A[r][v] B[c][v],
// A[tap][v] the 1-channel operand at the voxel's tap (BF16, K-major; row 27
// all ones, rows 28-127 zero), B the 32-channel operand at the tile's voxels
// (its 4 chunk planes, MN-major as the activation layout holds them):
//   input layer (MIRROR false): A = bf16(x) at v + s_tap, B = dZ1: dW_in, and
//     the ones row gives db_in;
//   output layer (MIRROR true): A = bf16(dy) at v - s_tap, B = A3: dW_out
//     (sum_v dy[v] A3[v + s_tap] = sum_u dy[u - s_tap] A3[u]).
// The accumulator stays in tensor memory over the CTA's tiles; each CTA
// writes its 28 x 32 partial sums (element-major: partial[e][cta]) and
// k_dn_wgrad1_reduce adds the CTAs' partials in a fixed order.
constexpr int kW1Threads = 128;
constexpr int kW1CtasPerSm = 4;
constexpr int kW1Rows = kTaps + 1;                    // 27 taps + the ones row
constexpr int kW1Partial = kW1Rows * kC;
constexpr int kW1ABytes = kTileM * kTileM * 2;       // A: 128 x 128 BF16
constexpr int kW1BBytes = 4 * kBodyBytes;            // B: 4 chunk planes of 128 voxels
constexpr int kW1Smem = 1024 + kW1ABytes + kW1BBytes + 9 * (kTileM + 2) * 4 + 64;
// A K-major (8-row groups 2048 B apart, K core matrices 128 B apart); B MN-major as in k_dn_wgrad_tc
constexpr uint64_t kAW1 = ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(2048 >> 4) << 32) | (1ull << 46);
constexpr uint64_t kBW1 = ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(kBodyBytes >> 4) << 32) | (1ull << 46);
constexpr uint32_t kIdescW1 = kIdescM128 | (4u << 17) | (1u << 16);  // N = 32, B MN-major

__device__ __forceinline__ uint32_t w1_a_offset(int row, int v) {
    return (uint32_t)((row >> 3) * 2048 + (v >> 3) * 128 + (row & 7) * 16 + (v & 7) * 2);
}

template <bool MIRROR>
__global__ void __launch_bounds__(kW1Threads) k_dn_wgrad1_tc(const float *__restrict__ s1,
                                                             const __nv_bfloat16 *__restrict__ S32,
                                                             float *__restrict__ partial, Dims d,
                                                             unsigned *__restrict__ err) {
    extern __shared__ uint8_t smem_raw[];
    const uint32_t raw = smem_u32(smem_raw);
    const uint32_t sA0 = (raw + 1023u) & ~1023u;
    uint8_t *const sA = smem_raw + (sA0 - raw);
    const uint32_t sB0 = sA0 + kW1ABytes;
    float *const sx = reinterpret_cast<float *>(sA + kW1ABytes + kW1BBytes);  // 9 lines x (128 + 2)
    const uint32_t mb = sB0 + kW1BBytes + 9 * (kTileM + 2) * 4;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(sA + (mb - sA0) + 8);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // rows 27 .. 127 of A once: the ones row, then zeros
    for (int i = tid; i < (kTileM - kTaps) * kTileM; i += kW1Threads) {
        const int row = kTaps + i / kTileM, v = i % kTileM;
        *reinterpret_cast<__nv_bfloat16 *>(sA + w1_a_offset(row, v)) =
            __float2bfloat16_rn(row == kTaps ? 1.f : 0.f);
    }
    if (tid == 0) {
        mbar_init(mb, 1);
        fence_mbar_init();
    }
    if (warp == 0) tmem_alloc(smem_u32(tslot), 32);
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    const uint32_t tmem = *tslot;
    const uint64_t adesc = kAW1 | (uint64_t)((sA0 >> 4) & 0x3FFFu);
    const uint64_t bdesc = kBW1 | (uint64_t)((sB0 >> 4) & 0x3FFFu);
    const int nseg = d.ny / kTileM, T = d.nx * d.np * nseg;
    uint32_t phase = 0, acc = 0;
    bool ok = true;
    for (int t = blockIdx.x; t < T && ok; t += gridDim.x) {
        const int p = t % d.np, y0 = ((t / d.np) % nseg) * kTileM, xx = t / (d.np * nseg);
        // the 1-channel operand's 9 lines (dx, dphi) over y0 - 1 .. y0 + 128
        for (int i = tid; i < 9 * (kTileM + 2); i += kW1Threads) {
            const int ys = i % (kTileM + 2), l = i / (kTileM + 2);
            const int gx = wrap_idx(xx + l / 3 - 1, d.nx), gp = wrap_idx(p + l % 3 - 1, d.np);
            sx[l * (kTileM + 2) + ys] = s1[((size_t)gx * d.np + gp) * d.ny + wrap_idx(y0 + ys - 1, d.ny)];
        }
        // B: the 32-channel operand's 4 chunk planes at the tile's voxels
        const size_t line = (size_t)xx * d.np + p;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const uint4 u = *reinterpret_cast<const uint4 *>(S32 + ((line * 4 + c) * d.ny + y0 + tid) * 8);
            st_shared16(sB0 + (uint32_t)(c * kBodyBytes + tid * 16), u);
        }
        __syncthreads();
        // A rows 0 .. 26, column tid: tap k = 9 dx + 3 dy + dphi
#pragma unroll
        for (int k = 0; k < kTaps; ++k) {
            const int dx = k / 9, dy = (k / 3) % 3, dp = k % 3;
            const float v = MIRROR ? sx[((2 - dx) * 3 + (2 - dp)) * (kTileM + 2) + tid + 2 - dy]
                                   : sx[(dx * 3 + dp) * (kTileM + 2) + tid + dy];
            *reinterpret_cast<__nv_bfloat16 *>(sA + w1_a_offset(k, tid)) = __float2bfloat16_rn(v);
        }
        fence_proxy_async();  // A and B, written by the threads, are read by the tensor core
        __syncthreads();
        if (tid == 0) {
            tc_after_sync();
#pragma unroll
            for (int kk = 0; kk < kTileM / 16; ++kk) {
                mma_bf16(tmem, adesc + (uint64_t)(kk * 256 >> 4), bdesc + (uint64_t)(kk * 256 >> 4), kIdescW1, acc);
                acc = 1u;
            }
            mma_commit(mb);
        }
        acc = 1u;
        ok = __syncthreads_and(mbar_wait(mb, phase));
        phase ^= 1u;
    }
    if (!ok && tid == 0) {
        atomicOr(err, kErrTimeout);
        mbar_wait(mb, phase ^ 1u);  // an MMA still in flight completes before the tensor memory is freed
    }
    tc_after_sync();
    if (warp == 0) {  // rows 0 .. 27 lie in tensor-memory lanes 0 .. 27
        uint32_t r[32];
        tmem_ld32(tmem, r);
        if (lane < kW1Rows) {
            const bool any = (int)blockIdx.x < T;  // a CTA without tiles leaves its accumulator unwritten
#pragma unroll
            for (int c = 0; c < kC; ++c)
                partial[(size_t)(lane * kC + c) * gridDim.x + blockIdx.x] = any ? __uint_as_float(r[c]) : 0.f;
        }
    }
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    if (warp == 0) tmem_dealloc(tmem, 32);
}

// dW[e] (e < 27 x 32) and db[e - 864] (the ones row) += the sum over the CTAs
// of partial[e][cta]: one warp per element, lane l adding the CTAs l, l + 32,
// ... in order, then a fixed shuffle tree (the same order every run)
__global__ void k_dn_wgrad1_reduce(const float *__restrict__ partial, int ncta, float *__restrict__ dW,
                                   float *__restrict__ db) {
    const int e = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (e >= kW1Partial) return;
    float s = 0.f;
    for (int c = lane; c < ncta; c += 32) s += partial[(size_t)e * ncta + c];
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) {
        if (e < kTaps * kC) dW[e] += s;
        else if (db) db[e - kTaps * kC] += s;
    }
}

// dW[e] += sum over the CTAs c of partial[c][e], in the order c = 0, 1, ...
// (e < 27 x 32 x 32: the weights, then the 32 biases)
__global__ void k_dn_wgrad_reduce(const float *__restrict__ partial, int ncta, float *__restrict__ dW,
                                  float *__restrict__ db) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= kWgPartial) return;
    float s = 0.f;
    for (int c = 0; c < ncta; ++c) s += partial[(size_t)c * kWgPartial + e];
    if (e < kTaps * kC * kC) dW[e] += s;
    else db[e - kTaps * kC * kC] += s;
}

// FP32 weights W[tap][n][k] -> BF16 in the K-major core-matrix layout of the
// B operand, one 2 KB block per tap, tap = 9 (dx + 1) + 3 (dy + 1) + (dphi + 1);
// within each (dx, dy) triple the blocks run dphi = +1, 0, -1, so that the
// triple is the B operand of N = 96 whose column blocks feed the output
// tiles phi - 1, phi, phi + 1 of one input position.  MIRROR: tap t holds
// W[26 - t][k][n] (the weights of the backward-data convolution).
template <bool MIRROR>
__global__ void k_pack_weights(const float *__restrict__ W, uint8_t *__restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kTaps * kC * kC) return;
    const int t = i / (kC * kC), n = (i / kC) % kC, k = i % kC;
    const float w = MIRROR ? W[((kTaps - 1 - t) * kC + k) * kC + n] : W[(t * kC + n) * kC + k];
    const int block = t - t % 3 + (2 - t % 3);
    *reinterpret_cast<__nv_bfloat16 *>(out + block * kBTap + core_offset(n, k)) = __float2bfloat16_rn(w);
}

// the 1 -> 32 input layer's weights w[tap][co] as the B operand [32 co][32 taps]
// of its GEMM (taps 27-31 zero); MIRROR: tap k holds w[26 - k] (the output
// layer's weights for its backward through the same GEMM)
template <bool MIRROR>
__global__ void k_pack_in_weights(const float *__restrict__ W, uint8_t *__restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kC * kC) return;
    const int n = i / kC, k = i % kC;
    const float w = k < kTaps ? W[(MIRROR ? kTaps - 1 - k : k) * kC + n] : 0.f;
    *reinterpret_cast<__nv_bfloat16 *>(out + core_offset(n, k)) = __float2bfloat16_rn(w);
}

// the 32 -> 1 output layer's weights w[tap][ci] as the operand of output
// channel 0 of a 32 -> 32 layer (channels 1-31 zero)
__global__ void k_pack_out_weights(const float *__restrict__ W, uint8_t *__restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kTaps * kC * kC) return;
    const int t = i / (kC * kC), n = (i / kC) % kC, k = i % kC;
    const float w = n == 0 ? W[t * kC + k] : 0.f;
    const int block = t - t % 3 + (2 - t % 3);
    *reinterpret_cast<__nv_bfloat16 *>(out + block * kBTap + core_offset(n, k)) = __float2bfloat16_rn(w);
}

int g_sms = 0;

// tiles of the convolution: (x, y segment of 128, phi)
int conv_tiles(Dims d) { return d.nx * (d.ny / kTileM) * d.np; }
template <int MODE>
static void conv_dispatch(int sms, const __nv_bfloat16 *X, const uint8_t *W, const float *bias,
                          const __nv_bfloat16 *ref, const float *res, void *Y, Dims d, unsigned *err,
                          cudaStream_t s) {
    using CS = ConvShape<kConvRows>;
    const int tiles = ((d.nx + kConvRows - 1) / kConvRows) * (d.ny / kTileM) * d.np;
    const int grid = tiles < sms ? tiles : sms;
    k_conv32<MODE, kConvRows><<<grid, CS::kThreads, CS::kSmem, s>>>(X, W, bias, ref, res, Y, d, err);
}
static void conv_set_attrs() {
    const int smem = ConvShape<kConvRows>::kSmem;
    cudaFuncSetAttribute(k_conv32<0, kConvRows>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaFuncSetAttribute(k_conv32<1, kConvRows>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaFuncSetAttribute(k_conv32<2, kConvRows>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaFuncSetAttribute(k_conv32<3, kConvRows>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
}



// ---- the network's CUDA-core layers -----------------------------------
// Parameters (FP32, one array): w_in[27][32], b_in[32], w2[27][32][32],
// b2[32], w3[27][32][32], b3[32], w_out[27][32], b_out.
constexpr int kOffWin = 0, kOffBin = kOffWin + kTaps * kC, kOffW2 = kOffBin + kC, kOffB2 = kOffW2 + kTaps * kC * kC,
              kOffW3 = kOffB2 + kC, kOffB3 = kOffW3 + kTaps * kC * kC, kOffWout = kOffB3 + kC,
              kOffBout = kOffWout + kTaps * kC, kParams = kOffBout + 1;

// The activation layout: line = x np + phi, channel chunk c = channel / 8
// (16 B of BF16); element (line, y, channel) at ((line 4 + c) ny + y) 8 +
// channel % 8.  Each line's chunk plane (ny rows of 16 B) is contiguous, so
// a tile's 128 rows of one chunk are one 2 KB block.  act_at(v, c, ny) is
// the element offset of chunk c of voxel v = line ny + y.
__device__ __forceinline__ size_t act_at_line(uint32_t line, uint32_t y, int c, int ny) {
    return (((size_t)line * 4 + (size_t)c) * (size_t)ny + y) * 8;
}
__device__ __forceinline__ size_t act_at(size_t v, int c, int ny) {
    const uint32_t line = (uint32_t)v / (uint32_t)ny, y = (uint32_t)v - line * (uint32_t)ny;  // v < 2^27
    return act_at_line(line, y, c, ny);
}
// the 32 channels of voxel v, rounded to BF16
__device__ __forceinline__ void store_act32(__nv_bfloat16 *A, size_t v, int ny, const float (&a)[32]) {
    const size_t at0 = act_at(v, 0, ny), plane = (size_t)ny * 8;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        uint32_t q[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            __nv_bfloat162 h = __floats2bfloat162_rn(a[8 * c + 2 * i], a[8 * c + 2 * i + 1]);
            q[i] = *reinterpret_cast<uint32_t *>(&h);
        }
        *reinterpret_cast<uint4 *>(A + at0 + c * plane) = make_uint4(q[0], q[1], q[2], q[3]);
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

// ---- the input layer on the tensor cores --------------------------------
// Input layer 1 -> 32 channels with ReLU, A1[v] = ReLU(b_in + sum_tap
// w_in[tap] bf16(x[nbr(v, tap)])), as one GEMM per tile of 128 voxels (x,
// phi, y0 .. y0 + 127): A[128 voxels][32] holds the input at the voxel's 27
// taps (tap = 9 (dx+1) + 3 (dy+1) + (dphi+1)) in BF16, columns 27-31 zero;
// B = w_in as [32 out][32 taps]; D[128][32] in tensor memory (2 MMAs of
// K = 16).  A CTA of 128 threads stages the tile's 9 input lines with their
// periodic y halo in shared memory, each thread builds its voxel's row of A
// there (K-major core matrices), one thread issues the MMAs, and every warp
// reads its 32 rows of D back for the bias, the ReLU and the BF16 store.
// Several CTAs per SM overlap one another's staging, MMAs and stores.
// BWD: the output layer's backward into its input with the same GEMM,
// dZ3[u][c] = (sum_tap w_out[tap][c] dy[nbr(u, 26 - tap)]) * (A3[u][c] > 0):
// the input is dy, B the output weights at the mirrored taps (w_out[26 - k]
// for tap k), and the epilogue applies ReLU'(A3) (ref) instead of bias and ReLU.
constexpr int kInThreads = 128;
constexpr int kInCtasPerSm = 8;  // 8 x 32 tensor-memory columns per SM

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
    __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&h);
}

// (the backward's epilogue needs more registers: 6 blocks per SM instead of 8, no spills)
template <bool BWD>
__global__ void __launch_bounds__(kInThreads, BWD ? 6 : kInCtasPerSm) k_dn_in_tc(const float *__restrict__ x,
                                                         const uint8_t *__restrict__ Wpi,
                                                         const float *__restrict__ bias,
                                                         const __nv_bfloat16 *__restrict__ ref,
                                                         __nv_bfloat16 *__restrict__ A1, Dims d,
                                                         unsigned *__restrict__ err) {
    __shared__ __align__(1024) uint8_t sA[kTileM * kC * 2];  // [128][32] BF16, core matrices
    __shared__ __align__(1024) uint8_t sW[kC * kC * 2];      // [32][32] BF16, core matrices
    __shared__ float sx[9][kTileM + 2];                      // line (dx, dphi), rows y0 - 1 .. y0 + 128
    __shared__ float sb[kC];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tslot;
    const int tid = threadIdx.x, warp = tid >> 5;
    for (int i = tid; i < kC * kC * 2 / 16; i += kInThreads)
        reinterpret_cast<uint4 *>(sW)[i] = reinterpret_cast<const uint4 *>(Wpi)[i];
    if (!BWD && tid < kC) sb[tid] = bias[tid];
    const uint32_t mb = smem_u32(&mbar);
    if (tid == 0) {
        mbar_init(mb, 1);
        fence_mbar_init();
    }
    if (warp == 0) tmem_alloc(smem_u32(&tslot), 32);
    fence_proxy_async();  // the weights, written by the threads, are read by the tensor core
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    const uint32_t tmem = tslot;
    const uint64_t adesc = kBDesc | (uint64_t)((smem_u32(sA) >> 4) & 0x3FFFu);
    const uint64_t bdesc = kBDesc | (uint64_t)((smem_u32(sW) >> 4) & 0x3FFFu);
    constexpr uint32_t kIdesc = kIdescM128 | (4u << 17);  // N = 32
    const int nseg = d.ny / kTileM, T = d.nx * d.np * nseg;
    uint32_t phase = 0;
    bool ok = true;
    for (int t = blockIdx.x; t < T && ok; t += gridDim.x) {
        const int p = t % d.np, y0 = ((t / d.np) % nseg) * kTileM, xx = t / (d.np * nseg);
        for (int i = tid; i < 9 * (kTileM + 2); i += kInThreads) {
            const int ys = i % (kTileM + 2), l = i / (kTileM + 2);
            const int gx = wrap_idx(xx + l / 3 - 1, d.nx), gp = wrap_idx(p + l % 3 - 1, d.np);
            sx[l][ys] = x[((size_t)gx * d.np + gp) * d.ny + wrap_idx(y0 + ys - 1, d.ny)];
        }
        __syncthreads();
        // row tid of A: tap k = 9 dx + 3 dy + dphi reads line (dx, dphi) at row tid + dy
        uint32_t w[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            float v[2];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int k = 2 * j + h;
                v[h] = k < kTaps ? sx[(k / 9) * 3 + k % 3][tid + (k / 3) % 3] : 0.f;
            }
            w[j] = pack_bf16x2(v[0], v[1]);
        }
#pragma unroll
        for (int c = 0; c < 4; ++c)
            st_shared16(smem_u32(sA) + (uint32_t)core_offset(tid, 8 * c),
                        make_uint4(w[4 * c], w[4 * c + 1], w[4 * c + 2], w[4 * c + 3]));
        fence_proxy_async();  // the rows of A, written by the threads, are read by the tensor core
        __syncthreads();
        if (tid == 0) {
            tc_after_sync();
            mma_bf16(tmem, adesc, bdesc, kIdesc, 0u);
            mma_bf16(tmem, adesc + (256 >> 4), bdesc + (256 >> 4), kIdesc, 1u);  // taps 16 .. 31
            mma_commit(mb);
        }
        ok = __syncthreads_and(mbar_wait(mb, phase));
        phase ^= 1u;
        if (!ok) break;
        tc_after_sync();
        uint32_t r[32];
        tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16), r);  // warp w: rows (voxels) 32 w ..
        tc_before_sync();
        float a[32];
        const size_t line = (size_t)xx * d.np + p;
        if (BWD) {
            // ReLU'(A3) at this voxel: its 4 chunk planes, two BF16 channels per word
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const uint4 u = *reinterpret_cast<const uint4 *>(ref + ((line * 4 + c) * d.ny + y0 + tid) * 8);
                const uint32_t w4[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    a[8 * c + 2 * j] = __uint_as_float(w4[j] << 16) > 0.f ? __uint_as_float(r[8 * c + 2 * j]) : 0.f;
                    a[8 * c + 2 * j + 1] =
                        __uint_as_float(w4[j] & 0xFFFF0000u) > 0.f ? __uint_as_float(r[8 * c + 2 * j + 1]) : 0.f;
                }
            }
        } else {
#pragma unroll
            for (int c = 0; c < kC; ++c) a[c] = fmaxf(__uint_as_float(r[c]) + sb[c], 0.f);
        }
        store_act32(A1, line * d.ny + y0 + tid, d.ny, a);
    }
    if (!ok && tid == 0) {
        atomicOr(err, kErrTimeout);
        // an MMA still in flight completes before the tensor memory is freed
        mbar_wait(mb, phase ^ 1u);
    }
    __syncthreads();
    tc_after_sync();
    if (warp == 0) tmem_dealloc(tmem, 32);
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
        ny % kTileM != 0 || (unsigned long long)nx * ny * np > (1ull << 27) ||
        (((uintptr_t)x | (uintptr_t)y | (uintptr_t)ref) & 15u) != 0) {
        ss::record_error(
            "ss_dn_conv32: null pointer, mode > 2, ny not a positive multiple of 128, or x, y, ref not 16-byte "
            "aligned");
        return SS_ERR_INVALID_ARGUMENT;
    }
    Dims d{(int)nx, (int)ny, (int)np};
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaSuccess;
    if (!g_sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
        if (g_sms <= 0) g_sms = 1;
        conv_set_attrs();
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
        const __nv_bfloat16 *X = reinterpret_cast<const __nv_bfloat16 *>(x);
        const __nv_bfloat16 *R = reinterpret_cast<const __nv_bfloat16 *>(ref);
        if (mode == 0) conv_dispatch<0>(g_sms, X, packed, bias, R, nullptr, y, d, derr, s);
        else if (mode == 1) conv_dispatch<1>(g_sms, X, packed, bias, R, nullptr, y, d, derr, s);
        else conv_dispatch<2>(g_sms, X, packed, bias, R, nullptr, y, d, derr, s);
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
    uint8_t *Wp2 = nullptr, *Wp3 = nullptr, *Wm2 = nullptr, *Wm3 = nullptr, *Wpo = nullptr, *Wpi = nullptr, *Wpob = nullptr;
    __nv_bfloat16 *A1 = nullptr, *A2 = nullptr, *A3 = nullptr, *D1 = nullptr, *D2 = nullptr;
    float *wpart = nullptr;  // the weight gradients' per-CTA partial sums
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
    conv_set_attrs();
    cudaFuncSetAttribute(k_dn_wgrad_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemWg);
    done = true;
}

template <int MODE>
void launch_conv(ss_dn *n, const __nv_bfloat16 *X, const uint8_t *W, const float *bias, const __nv_bfloat16 *ref,
                 void *Y, cudaStream_t s, const float *res = nullptr) {
    conv_dispatch<MODE>(n->sms, X, W, bias, ref, res, Y, n->d, n->err, s);
}

void pack_all(ss_dn *n, cudaStream_t s) {
    const int nw = kTaps * kC * kC, b = (nw + 255) / 256;
    k_pack_weights<false><<<b, 256, 0, s>>>(n->P + kOffW2, n->Wp2);
    k_pack_weights<false><<<b, 256, 0, s>>>(n->P + kOffW3, n->Wp3);
    k_pack_weights<true><<<b, 256, 0, s>>>(n->P + kOffW2, n->Wm2);
    k_pack_weights<true><<<b, 256, 0, s>>>(n->P + kOffW3, n->Wm3);
    k_pack_out_weights<<<b, 256, 0, s>>>(n->P + kOffWout, n->Wpo);
    k_pack_in_weights<false><<<(kC * kC + 255) / 256, 256, 0, s>>>(n->P + kOffWin, n->Wpi);
    k_pack_in_weights<true><<<(kC * kC + 255) / 256, 256, 0, s>>>(n->P + kOffWout, n->Wpob);
    n->launches += 7;
}

template <bool TO_ACT>
void transpose(ss_dn *n, const float *src, float *dst, cudaStream_t s) {
    const int R = TO_ACT ? n->d.ny : n->d.np, Cn = TO_ACT ? n->d.np : n->d.ny;
    k_dn_transpose<TO_ACT><<<dim3((Cn + 31) / 32, (R + 31) / 32, n->d.nx), dim3(32, 8), 0, s>>>(src, dst, n->d);
}

// the network on x (histogram layout), output ya in the activation layout
void enqueue_forward_act(ss_dn *n, const float *x, float *ya, cudaStream_t s) {
    transpose<true>(n, x, n->xa, s);
    const int tiles = n->d.nx * n->d.np * (n->d.ny / kTileM), in_grid = tiles < kInCtasPerSm * n->sms ? tiles : kInCtasPerSm * n->sms;
    k_dn_in_tc<false><<<in_grid, kInThreads, 0, s>>>(n->xa, n->Wpi, n->P + kOffBin, nullptr, n->A1, n->d, n->err);
    launch_conv<0>(n, n->A1, n->Wp2, n->P + kOffB2, nullptr, n->A2, s);
    launch_conv<0>(n, n->A2, n->Wp3, n->P + kOffB3, nullptr, n->A3, s);
    // the 32 -> 1 output layer on the tensor cores (BF16 weights), + the residual
    launch_conv<3>(n, n->A3, n->Wpo, n->P + kOffBout, nullptr, ya, s, n->xa);
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
    transpose<true>(n, t, n->ta, s);
    if (n->moment_weight > 0.f)
        k_dn_loss_moment<<<2 * n->sms, 128, 2 * n->d.np * sizeof(float), s>>>(
            ya, n->ta, n->dy, n->d, n->moment_weight, n->sums, grads ? n->G + kOffBout : nullptr);
    else
        k_dn_loss<<<2 * n->sms, 256, 0, s>>>(ya, n->ta, n->dy, n->nvox, n->sums, grads ? n->G + kOffBout : nullptr);
    n->launches += 2;
    if (!grads) return;
    const int wgrid = conv_tiles(n->d) < n->sms ? conv_tiles(n->d) : n->sms;
    auto wgrad = [&](const __nv_bfloat16 *dZ, const __nv_bfloat16 *A, float *dW, float *db) {
        k_dn_wgrad_tc<<<wgrid, kWgThreads, kSmemWg, s>>>(dZ, A, n->wpart, n->d, n->err);
        k_dn_wgrad_reduce<<<(kWgPartial + 255) / 256, 256, 0, s>>>(n->wpart, wgrid, dW, db);
    };
    // the 1-channel layers' weight gradients on the tensor cores, fixed-order sums over the CTAs
    const int w1grid = n->ntiles < kW1CtasPerSm * n->sms ? n->ntiles : kW1CtasPerSm * n->sms;
    auto wgrad1 = [&](bool out_layer, float *dW, float *db) {
        if (out_layer) k_dn_wgrad1_tc<true><<<w1grid, kW1Threads, kW1Smem, s>>>(n->dy, n->A3, n->wpart, n->d, n->err);
        else k_dn_wgrad1_tc<false><<<w1grid, kW1Threads, kW1Smem, s>>>(n->xa, n->D1, n->wpart, n->d, n->err);
        k_dn_wgrad1_reduce<<<(kW1Partial * 32 + 255) / 256, 256, 0, s>>>(n->wpart, w1grid, dW, db);
    };
    // the output layer's backward into dZ3 (in D1): the input layer's GEMM on dy with mirrored weights
    const int tiles = n->d.nx * n->d.np * (n->d.ny / kTileM), in_grid = tiles < kInCtasPerSm * n->sms ? tiles : kInCtasPerSm * n->sms;
    k_dn_in_tc<true><<<in_grid, kInThreads, 0, s>>>(n->dy, n->Wpob, nullptr, n->A3, n->D1, n->d, n->err);
    wgrad1(true, n->G + kOffWout, nullptr);
    wgrad(n->D1, n->A2, n->G + kOffW3, n->G + kOffB3);
    launch_conv<2>(n, n->D1, n->Wm3, nullptr, n->A2, n->D2, s);
    wgrad(n->D2, n->A1, n->G + kOffW2, n->G + kOffB2);
    launch_conv<2>(n, n->D2, n->Wm2, nullptr, n->A1, n->D1, s);
    wgrad1(false, n->G + kOffWin, n->G + kOffBin);
    n->launches += 12;
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
    cudaFree(n->Wp2); cudaFree(n->Wp3); cudaFree(n->Wm2); cudaFree(n->Wm3); cudaFree(n->Wpo); cudaFree(n->Wpi); cudaFree(n->Wpob);
    cudaFree(n->A1); cudaFree(n->A2); cudaFree(n->A3); cudaFree(n->D1); cudaFree(n->D2);
    cudaFree(n->sums); cudaFree(n->err); cudaFree(n->wpart);
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
    A((void **)&n->Wpo, kBAll);
    A((void **)&n->Wpi, kC * kC * 2);
    A((void **)&n->Wpob, kC * kC * 2);
    A((void **)&n->A1, ab); A((void **)&n->A2, ab); A((void **)&n->A3, ab); A((void **)&n->D1, ab);
    A((void **)&n->D2, ab);
    A((void **)&n->sums, 2 * sizeof(double)); A((void **)&n->err, sizeof(unsigned));
    A((void **)&n->wpart, (size_t)(n->sms > 0 ? n->sms : 1) * kWgPartial * sizeof(float));
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
