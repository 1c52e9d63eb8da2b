// denoiser.cu -- the learned histogram denoiser: a 3-D CNN (4 convolutions
// of 3x3x3 with periodic padding, 32 channels, ReLU, residual) that maps a
// low-particle-count histogram on the (x, y, phi) grid to an estimate of the
// high-count distribution before the stress / Stokes solve.
//
// The 32 -> 32 convolutions are implicit GEMMs on the 5th-generation tensor
// cores: per tile of 128 voxels, D[128 x 32] = sum over the 27 taps of
// A_tap[128 x 32] * W_tap[32 x 32]^T with BF16 operands and an FP32
// accumulator in tensor memory.  One elected thread issues tcgen05.mma
// (M = 128, N = 32, K = 16, two per tap); the A rows of a tap (the periodic
// neighbours of the tile's voxels, 64 bytes each, channels-last) are copied
// into shared memory with cp.async into a 4-stage ring whose reuse is gated
// by mbarriers that tcgen05.commit arrives on; the 27 weight taps stay in
// shared memory for the whole persistent CTA.  The epilogue reads the
// accumulator with tcgen05.ld (one voxel's 32 channels per thread), adds the
// bias and applies ReLU (or the ReLU derivative of a reference tensor for
// the backward pass) and stores channels-last.
//
// Shared-memory operand layout (K-major, no swizzle): core matrices of 8 rows
// x 16 bytes; the 4 core matrices of a row group along K are contiguous
// (leading-dimension offset 128 B), row groups are 512 B apart (stride
// offset).  Every wait is bounded: on a timeout the kernel records an error,
// waits for its own copies, frees its tensor memory and returns.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>

#include "../../include/ssgpu.h"

namespace ss {
void record_error(const char *msg);
}

namespace {

constexpr int kC = 32;                       // channels
constexpr int kTaps = 27;                    // 3 x 3 x 3
constexpr int kTileM = 128;                  // voxels per tile (MMA M)
constexpr int kStages = 4;                   // A ring
constexpr int kAStage = kTileM * kC * 2;     // 8 KB
constexpr int kBTap = kC * kC * 2;           // 2 KB
constexpr int kBAll = kTaps * kBTap;         // 54 KB
constexpr int kSmemConv = kBAll + kStages * kAStage + 128;
constexpr uint32_t kWaitLimit = 1u << 22;    // mbarrier polls before giving up
constexpr unsigned kErrTimeout = 1u;

struct Dims {
    int nx, ny, np;
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// voxel (x, y, p) <-> linear index (x ny + y) np + p.  A voxel's periodic
// neighbour at tap = (dx + 1) 9 + (dy + 1) 3 + (dp + 1), from its
// coordinates decoded once.
struct Voxel {
    int x, y, p;
    __device__ __forceinline__ Voxel(int v, Dims d) : x(v / (d.np * d.ny)), y((v / d.np) % d.ny), p(v % d.np) {}
    __device__ __forceinline__ int neighbour(int tap, Dims d) const {
        int a = x + tap / 9 - 1, b = y + (tap / 3) % 3 - 1, c = p + tap % 3 - 1;
        a = a < 0 ? a + d.nx : (a >= d.nx ? a - d.nx : a);
        b = b < 0 ? b + d.ny : (b >= d.ny ? b - d.ny : b);
        c = c < 0 ? c + d.np : (c >= d.np ? c - d.np : c);
        return (a * d.ny + b) * d.np + c;
    }
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

// shared-memory matrix descriptor: K-major, no swizzle, LBO 128 B, SBO 512 B
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)(128u >> 4) << 16) | ((uint64_t)(512u >> 4) << 32) |
           (1ull << 46);
}
// instruction descriptor: D FP32, A and B BF16, both K-major, N = 32, M = 128
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kC >> 3) << 17) |
                            ((uint32_t)(kTileM >> 4) << 24);

// byte offset of element (row, k) of a K-major operand block in the core-matrix layout
__host__ __device__ __forceinline__ int core_offset(int row, int k) {
    return (row >> 3) * 512 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2;
}

// MODE 0: bias + ReLU -> BF16; MODE 1: bias -> FP32; MODE 2: times ReLU'(ref) -> BF16
template <int MODE>
__global__ void __launch_bounds__(kTileM, 1) k_conv32(const __nv_bfloat16 *__restrict__ X,
                                                      const uint8_t *__restrict__ Wpacked,
                                                      const float *__restrict__ bias,
                                                      const __nv_bfloat16 *__restrict__ ref, void *__restrict__ Y,
                                                      Dims d, int ntiles, unsigned *__restrict__ err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t *sB = smem;
    uint8_t *sA = smem + kBAll;
    uint64_t *mbar = reinterpret_cast<uint64_t *>(sA + kStages * kAStage);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(mbar + kStages);
    volatile int *sfail = reinterpret_cast<volatile int *>(tslot + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    for (int i = tid; i < kBAll / 16; i += kTileM)
        reinterpret_cast<uint4 *>(sB)[i] = reinterpret_cast<const uint4 *>(Wpacked)[i];
    if (tid == 0) {
        for (int s = 0; s < kStages; ++s) mbar_init(smem_u32(&mbar[s]), 1);
        *sfail = 0;
        fence_mbar_init();
    }
    if (warp == 0) tmem_alloc(smem_u32(tslot), 32);
    fence_proxy_async();
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    const uint32_t tmem = *tslot;
    const uint32_t sA0 = smem_u32(sA), sB0 = smem_u32(sB);
    const int row_off = (tid >> 3) * 512 + (tid & 7) * 16;  // this thread's row in an A stage

    uint32_t it = 0;  // taps issued by this CTA (ring position)
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const Voxel vx(tile * kTileM + tid, d);
        // copy the A rows of tap t into stage it % kStages, after the MMA
        // that last read that stage has completed
        auto load_tap = [&](int t, uint32_t pos) -> bool {
            const uint32_t s = pos % kStages;
            if (pos >= kStages && !mbar_wait(smem_u32(&mbar[s]), ((pos - kStages) / kStages) & 1u)) return false;
            const uint8_t *src = reinterpret_cast<const uint8_t *>(X + (size_t)vx.neighbour(t, d) * kC);
            const uint32_t dst = sA0 + s * kAStage + row_off;
#pragma unroll
            for (int j = 0; j < 4; ++j) cp_async16(dst + j * 128, src + j * 16);
            return true;
        };
        bool ok = load_tap(0, it);
        cp_async_commit();
        for (int t = 0; t < kTaps; ++t) {
            if (t + 1 < kTaps) {
                ok = load_tap(t + 1, it + 1) && ok;
                cp_async_commit();
                cp_async_wait<1>();
            } else {
                cp_async_wait<0>();
            }
            if (!ok) *sfail = 1;
            fence_proxy_async();
            __syncthreads();
            if (*sfail) break;
            if (tid == 0) {
                tc_after_sync();
                const uint32_t s = it % kStages;
#pragma unroll
                for (int kk = 0; kk < 2; ++kk) {
                    const uint64_t ad = smem_desc(sA0 + s * kAStage + kk * 256);
                    const uint64_t bd = smem_desc(sB0 + t * kBTap + kk * 256);
                    mma_bf16(tmem, ad, bd, kIdesc, (t > 0 || kk > 0) ? 1u : 0u);
                }
                mma_commit(smem_u32(&mbar[s]));
            }
            ++it;
        }
        __syncthreads();
        if (*sfail) break;
        // the accumulator is complete when the tile's last MMA has completed
        const uint32_t last = it - 1;
        if (!mbar_wait(smem_u32(&mbar[last % kStages]), (last / kStages) & 1u)) *sfail = 1;
        __syncthreads();
        if (*sfail) break;
        tc_after_sync();
        uint32_t r[32];
        tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16), r);
        const int vo = tile * kTileM + warp * 32 + lane;  // this thread's accumulator row
        if (MODE == 1) {
            float4 *out = reinterpret_cast<float4 *>(reinterpret_cast<float *>(Y) + (size_t)vo * kC);
#pragma unroll
            for (int q = 0; q < 8; ++q)
                out[q] = make_float4(__uint_as_float(r[4 * q]) + bias[4 * q], __uint_as_float(r[4 * q + 1]) + bias[4 * q + 1],
                                     __uint_as_float(r[4 * q + 2]) + bias[4 * q + 2],
                                     __uint_as_float(r[4 * q + 3]) + bias[4 * q + 3]);
        } else {
            uint32_t packed[16];
            const __nv_bfloat16 *rr = ref + (size_t)vo * kC;
#pragma unroll
            for (int q = 0; q < 16; ++q) {
                float a = __uint_as_float(r[2 * q]), b = __uint_as_float(r[2 * q + 1]);
                if (MODE == 0) {
                    a = fmaxf(a + bias[2 * q], 0.f);
                    b = fmaxf(b + bias[2 * q + 1], 0.f);
                } else {
                    a = __bfloat162float(rr[2 * q]) > 0.f ? a : 0.f;
                    b = __bfloat162float(rr[2 * q + 1]) > 0.f ? b : 0.f;
                }
                __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
                packed[q] = *reinterpret_cast<uint32_t *>(&h);
            }
            uint4 *out = reinterpret_cast<uint4 *>(reinterpret_cast<__nv_bfloat16 *>(Y) + (size_t)vo * kC);
#pragma unroll
            for (int q = 0; q < 4; ++q)
                out[q] = make_uint4(packed[4 * q], packed[4 * q + 1], packed[4 * q + 2], packed[4 * q + 3]);
        }
        // every thread's tensor-memory reads finish before the next tile's MMAs overwrite it
        tc_before_sync();
        __syncthreads();
    }
    if (*sfail && tid == 0) atomicOr(err, kErrTimeout);
    cp_async_wait<0>();
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    if (warp == 0) tmem_dealloc(tmem, 32);
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

}  // namespace

extern "C" int ss_dn_conv32(const void *x, const float *w, const float *bias, const void *ref, void *y,
                            uint32_t nx, uint32_t ny, uint32_t np, uint32_t mode, void *stream) {
    char buf[256];
    if (!x || !w || !y || (mode != 2 && !bias) || (mode == 2 && !ref) || mode > 2 || nx < 1 || ny < 1 || np < 1 ||
        ((unsigned long long)nx * ny * np) % kTileM != 0 || (unsigned long long)nx * ny * np > (1ull << 30)) {
        ss::record_error("ss_dn_conv32: null pointer, mode > 2, or voxel count not a positive multiple of 128");
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
        const int ntiles = (int)(((unsigned long long)nx * ny * np) / kTileM);
        const int grid = ntiles < 2 * g_sms ? ntiles : 2 * g_sms;
        Dims d{(int)nx, (int)ny, (int)np};
        const __nv_bfloat16 *X = reinterpret_cast<const __nv_bfloat16 *>(x);
        const __nv_bfloat16 *R = reinterpret_cast<const __nv_bfloat16 *>(ref);
        if (mode == 0) k_conv32<0><<<grid, kTileM, kSmemConv, s>>>(X, packed, bias, R, y, d, ntiles, derr);
        else if (mode == 1) k_conv32<1><<<grid, kTileM, kSmemConv, s>>>(X, packed, bias, R, y, d, ntiles, derr);
        else k_conv32<2><<<grid, kTileM, kSmemConv, s>>>(X, packed, bias, R, y, d, ntiles, derr);
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
