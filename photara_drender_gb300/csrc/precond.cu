// Learned refine preconditioner: a 16 -> 64 -> 64 -> 4 MLP evaluated per atlas texel on the
// fifth-generation tensor cores, plus the kernels that feed it and apply it.
//
// GEMMs. A tile is 128 samples (the MMA's M, one TMEM lane per sample). Operands are BF16 in shared
// memory in the canonical K-major layout without swizzle: 8-row x 16-byte core matrices, K-adjacent
// core matrices 128 bytes apart (leading byte offset), 8-row groups K*16 bytes apart (stride byte
// offset). One elected thread issues tcgen05.mma (kind::f16, FP32 accumulate into TMEM) and commits
// to an mbarrier; each warp then reads its 32 TMEM lanes (its 32 samples) with tcgen05.ld, applies
// bias and ReLU in registers, and writes the next layer's operand back to shared memory.
//   forward:  D1 = X W1^T (K 16), D2 = H1 W2^T (K 64), D3 = H2 W3^T (K 64, N padded 4 -> 16)
//   training: the same forward, then dH2 = dY W3 (K 16) and dH1 = dZ2 W2 (K 64) on the tensor cores;
//             the weight gradients (outer products over the 128 samples; M <= 64, below the 128-row
//             MMA tile) are FP32 FMAs on the CUDA cores, accumulated per CTA and added once.
// Waits on the mbarrier give up after about a second: the kernel records PDR_STATUS_PRECOND_TIMEOUT,
// waits once more (bounded) for the MMA in flight, frees its TMEM and returns.
//
// Parameters live in one FP32 vector of PDR_PRECOND_PARAMS values [W1 64x16 | b1 | W2 64x64 | b2 |
// W3 4x64 | b3] (weights row-major [out][in]) with a BF16 copy of the same vector for the MMAs.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/pdr_capi.h"
#include "pdr_common.cuh"
#include "pdr_internal.h"

namespace pdr {
namespace {

constexpr uint32_t kIn = PDR_PRECOND_IN, kHid = PDR_PRECOND_HIDDEN, kOut = PDR_PRECOND_OUT;
constexpr uint32_t kOutPad = 16;    // the last layer runs with N = 16, the smallest N of an M = 128 MMA
constexpr uint32_t kRows = 128;     // samples per tile = MMA M = TMEM lanes
constexpr uint32_t kThreads = 128;  // warp w owns TMEM lanes 32w..32w+31
constexpr uint32_t kTrainCols = 128; // training: D1 / D3 / dH1 in columns 0..63, D2 / dH2 in 64..127
constexpr uint32_t kFwdCols = 64;    // inference: every layer's accumulator in columns 0..63
constexpr uint32_t kOffW1 = 0, kOffB1 = 1024, kOffW2 = 1088, kOffB2 = 5184, kOffW3 = 5248, kOffB3 = 5504;
static_assert(kOffB3 + kOut == PDR_PRECOND_PARAMS, "parameter layout");
constexpr long long kWaitCycles = 2000000000ll;  // about one second at 2 GHz

// ---- tcgen05 / mbarrier helpers -------------------------------------------------------------------

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// byte offset of element (row, k) of a K-column operand in the canonical no-swizzle K-major layout
__device__ __forceinline__ uint32_t core_off(uint32_t row, uint32_t k, uint32_t K) {
    return (row >> 3) * (K * 16u) + (k >> 3) * 128u + (row & 7u) * 16u + (k & 7u) * 2u;
}

// shared-memory matrix descriptor: start address, leading byte offset 128 (next core matrix along K),
// stride byte offset K*16 (next 8-row group), descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t operand_desc(uint32_t addr, uint32_t K) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(128u >> 4) << 16) | ((uint64_t)((K * 16u) >> 4) << 32) |
           (1ull << 46);
}

// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major, N >> 3, M >> 4
constexpr uint32_t idesc_bf16(uint32_t M, uint32_t N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.u32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}

// true once the mbarrier phase of the given parity has completed; false after about a second
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
    const long long t0 = clock64();
    while (true) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
        if (clock64() - t0 > kWaitCycles) return false;
    }
}

__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }

// shared-memory writes by this thread become visible to the tensor cores, then the CTA meets
__device__ __forceinline__ void operands_ready() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    fence_before_sync();
    __syncthreads();
}

// 16 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        "tcgen05.wait::ld.sync.aligned;\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// 64 consecutive FP32 columns of this thread's TMEM lane (load and wait in one statement, so no use of
// the registers can be scheduled before the data has arrived)
__device__ __forceinline__ void tmem_ld64(uint32_t taddr, float* v) {
    uint32_t r[64];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x64.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47,%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, [%64];\n"
        "tcgen05.wait::ld.sync.aligned;\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]), "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]), "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]), "=r"(r[48]), "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]), "=r"(r[56]), "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 64; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&h);
}

__device__ __forceinline__ float bf16_lo(uint32_t w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t w) { return __uint_as_float(w & 0xffff0000u); }

// 16 values (columns c0..c0+15) of row `row` into a K-column BF16 operand: two 16-byte stores
__device__ __forceinline__ void store_row16(uint8_t* base, uint32_t row, uint32_t c0, uint32_t K, const float* v) {
    uint4 a, b;
    a.x = pack_bf16(v[0], v[1]);
    a.y = pack_bf16(v[2], v[3]);
    a.z = pack_bf16(v[4], v[5]);
    a.w = pack_bf16(v[6], v[7]);
    b.x = pack_bf16(v[8], v[9]);
    b.y = pack_bf16(v[10], v[11]);
    b.z = pack_bf16(v[12], v[13]);
    b.w = pack_bf16(v[14], v[15]);
    *reinterpret_cast<uint4*>(base + core_off(row, c0, K)) = a;
    *reinterpret_cast<uint4*>(base + core_off(row, c0 + 8, K)) = b;
}

// Weights of one layer, row-major [rows][K] BF16 in global memory, into the K-major operand layout;
// rows >= valid_rows are zero.
__device__ __forceinline__ void load_weight(uint8_t* dst, const __nv_bfloat16* src, uint32_t rows, uint32_t valid_rows,
                                            uint32_t K) {
    const uint32_t chunks = rows * (K / 8);
    for (uint32_t c = threadIdx.x; c < chunks; c += blockDim.x) {
        const uint32_t r = c / (K / 8), kc = c % (K / 8);
        uint4 v = make_uint4(0, 0, 0, 0);
        if (r < valid_rows) v = *reinterpret_cast<const uint4*>(src + (size_t)r * K + kc * 8);
        *reinterpret_cast<uint4*>(dst + core_off(r, kc * 8, K)) = v;
    }
}

// Transposed weights: operand element (n, k) = W[k][n] of a row-major [k_valid][N] matrix.
__device__ __forceinline__ void load_weight_t(uint8_t* dst, const __nv_bfloat16* src, uint32_t N, uint32_t K,
                                              uint32_t k_valid) {
    for (uint32_t e = threadIdx.x; e < N * K; e += blockDim.x) {
        const uint32_t n = e / K, k = e % K;
        const __nv_bfloat16 v = k < k_valid ? src[(size_t)k * N + n] : __float2bfloat16(0.0f);
        *reinterpret_cast<__nv_bfloat16*>(dst + core_off(n, k, K)) = v;
    }
}

struct TensorCoreCta {
    uint64_t mbar;
    uint32_t tmem;
    uint32_t abort;
};

__device__ __forceinline__ void tc_setup(TensorCoreCta& c, uint32_t cols) {
    if ((threadIdx.x >> 5) == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&c.tmem)),
                     "r"(cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&c.mbar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        c.abort = 0;
    }
}

// Thread 0 issues `slices` K=16 MMAs D (+)= A B^T and commits; every thread waits for completion.
// Returns false (and marks the CTA aborted) when the wait ran out.
__device__ __forceinline__ bool tc_gemm(TensorCoreCta& c, uint32_t d_col, uint32_t a_addr, uint32_t b_addr,
                                        uint32_t K, uint32_t slices, uint32_t idesc, uint32_t& phase) {
    if (threadIdx.x == 0) {
        fence_after_sync();
#pragma unroll 1
        for (uint32_t j = 0; j < slices; ++j)
            mma_bf16(c.tmem + d_col, operand_desc(a_addr + j * 256u, K), operand_desc(b_addr + j * 256u, K), idesc, j);
        mma_commit(smem_addr(&c.mbar));
    }
    const bool ok = mbar_wait(smem_addr(&c.mbar), phase);
    if (ok) phase ^= 1u;
    fence_after_sync();
    if (!ok) atomicOr(&c.abort, 1u);
    __syncthreads();
    return c.abort == 0;
}

__device__ __forceinline__ void tc_teardown(TensorCoreCta& c, uint32_t phase, uint32_t* status, uint32_t cols) {
    if (c.abort) {
        // the MMA of the current phase may still be running: wait for it once more before freeing TMEM
        mbar_wait(smem_addr(&c.mbar), phase);
        if (threadIdx.x == 0) atomicMax(status + PDR_STATUS_PRECOND_TIMEOUT, 1u);
    }
    fence_before_sync();
    __syncthreads();
    if ((threadIdx.x >> 5) == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(c.tmem), "r"(cols) : "memory");
}

constexpr uint32_t kIdescHid = idesc_bf16(kRows, kHid);
constexpr uint32_t kIdescOut = idesc_bf16(kRows, kOutPad);

// ---- inference ----------------------------------------------------------------------------------------

// The hidden activations of both layers share one buffer (layer 2's MMA has finished reading H1 before
// H2 is written), and every accumulator uses TMEM columns 0..63: about 32 KB of shared memory and 64
// columns per CTA, so up to seven tiles are in flight per SM.
struct __align__(128) FwdSmem {
    uint8_t x[kRows * kIn * 2];
    uint8_t h[kRows * kHid * 2];
    uint8_t w1[kHid * kIn * 2];
    uint8_t w2[kHid * kHid * 2];
    uint8_t w3[kOutPad * kHid * 2];
    float b1[kHid], b2[kHid], b3[kOutPad];
    TensorCoreCta tc;
};

__global__ void __launch_bounds__(kThreads) precond_forward_kernel(const float* __restrict__ params,
                                                                   const __nv_bfloat16* __restrict__ wbf,
                                                                   const __nv_bfloat16* __restrict__ feat, uint64_t n,
                                                                   float4* __restrict__ out,
                                                                   uint32_t* __restrict__ status) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    FwdSmem& s = *reinterpret_cast<FwdSmem*>(smem_raw);
    const uint32_t tid = threadIdx.x, warp = tid >> 5;
    tc_setup(s.tc, kFwdCols);
    load_weight(s.w1, wbf + kOffW1, kHid, kHid, kIn);
    load_weight(s.w2, wbf + kOffW2, kHid, kHid, kHid);
    load_weight(s.w3, wbf + kOffW3, kOutPad, kOut, kHid);
    for (uint32_t i = tid; i < kHid; i += kThreads) {
        s.b1[i] = params[kOffB1 + i];
        s.b2[i] = params[kOffB2 + i];
    }
    if (tid < kOutPad) s.b3[tid] = tid < kOut ? params[kOffB3 + tid] : 0.0f;
    operands_ready();
    fence_after_sync();
    const uint32_t lane_addr = (warp * 32u) << 16;
    uint32_t phase = 0;
    const uint64_t tiles = (n + kRows - 1) / kRows;
    for (uint64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const uint64_t row = tile * kRows + tid;
        uint4 f0 = make_uint4(0, 0, 0, 0), f1 = f0;
        if (row < n) {
            const uint4* src = reinterpret_cast<const uint4*>(feat + row * kIn);
            f0 = src[0];
            f1 = src[1];
        }
        *reinterpret_cast<uint4*>(s.x + core_off(tid, 0, kIn)) = f0;
        *reinterpret_cast<uint4*>(s.x + core_off(tid, 8, kIn)) = f1;
        operands_ready();
        if (!tc_gemm(s.tc, 0, smem_addr(s.x), smem_addr(s.w1), kIn, 1, kIdescHid, phase)) break;
        float v[64];
        tmem_ld64(s.tc.tmem + lane_addr, v);
#pragma unroll
        for (uint32_t c0 = 0; c0 < kHid; c0 += 16) {
#pragma unroll
            for (int i = 0; i < 16; ++i) v[c0 + i] = fmaxf(v[c0 + i] + s.b1[c0 + i], 0.0f);
            store_row16(s.h, tid, c0, kHid, v + c0);
        }
        operands_ready();
        if (!tc_gemm(s.tc, 0, smem_addr(s.h), smem_addr(s.w2), kHid, 4, kIdescHid, phase)) break;
        tmem_ld64(s.tc.tmem + lane_addr, v);
#pragma unroll
        for (uint32_t c0 = 0; c0 < kHid; c0 += 16) {
#pragma unroll
            for (int i = 0; i < 16; ++i) v[c0 + i] = fmaxf(v[c0 + i] + s.b2[c0 + i], 0.0f);
            store_row16(s.h, tid, c0, kHid, v + c0);
        }
        operands_ready();
        if (!tc_gemm(s.tc, 0, smem_addr(s.h), smem_addr(s.w3), kHid, 4, kIdescOut, phase)) break;
        tmem_ld16(s.tc.tmem + lane_addr, v);
        if (row < n) out[row] = make_float4(v[0] + s.b3[0], v[1] + s.b3[1], v[2] + s.b3[2], v[3] + s.b3[3]);
        fence_before_sync();
        __syncthreads();
    }
    tc_teardown(s.tc, phase, status, kFwdCols);
}

// ---- training ---------------------------------------------------------------------------------------

struct __align__(128) TrainSmem {
    uint8_t x[kRows * kIn * 2];
    uint8_t h1[kRows * kHid * 2];
    uint8_t h2[kRows * kHid * 2];
    uint8_t dy[kRows * kOutPad * 2];
    uint8_t dz2[kRows * kHid * 2];
    uint8_t w1[kHid * kIn * 2];
    uint8_t w2[kHid * kHid * 2];
    uint8_t w3[kOutPad * kHid * 2];
    uint8_t w2t[kHid * kHid * 2];     // operand (n = in, k = out) = W2[out][in]
    uint8_t w3t[kHid * kOutPad * 2];  // operand (n = in, k = out) = W3[out][in], out padded to 16
    float dz1f[kRows * kHid];
    float dz2f[kRows * kHid];
    float dyf[kRows * kOut];
    float b1[kHid], b2[kHid], b3[kOutPad];
    float red[kThreads / 32];
    TensorCoreCta tc;
};

__global__ void __launch_bounds__(kThreads, 1) precond_train_kernel(
    const float* __restrict__ params, const __nv_bfloat16* __restrict__ wbf, const __nv_bfloat16* __restrict__ feat,
    const float4* __restrict__ target, const float4* __restrict__ weight, uint64_t n, float inv_norm,
    float* __restrict__ grads, float* __restrict__ loss, uint32_t* __restrict__ status) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    TrainSmem& s = *reinterpret_cast<TrainSmem*>(smem_raw);
    const uint32_t tid = threadIdx.x, warp = tid >> 5;
    tc_setup(s.tc, kTrainCols);
    load_weight(s.w1, wbf + kOffW1, kHid, kHid, kIn);
    load_weight(s.w2, wbf + kOffW2, kHid, kHid, kHid);
    load_weight(s.w3, wbf + kOffW3, kOutPad, kOut, kHid);
    load_weight_t(s.w2t, wbf + kOffW2, kHid, kHid, kHid);
    load_weight_t(s.w3t, wbf + kOffW3, kHid, kOutPad, kOut);
    for (uint32_t i = tid; i < kHid; i += kThreads) {
        s.b1[i] = params[kOffB1 + i];
        s.b2[i] = params[kOffB2 + i];
    }
    if (tid < kOutPad) s.b3[tid] = tid < kOut ? params[kOffB3 + tid] : 0.0f;
    operands_ready();
    fence_after_sync();

    // per-thread gradient accumulators: dW2 rows o = tid/2, columns (tid&1)*32 + 0..31; dW1 row tid/2,
    // columns (tid&1)*8 + 0..7; dW3 row tid/32, columns (tid&31)*2 + 0..1; b1 (tid < 64) / b2 (tid >= 64)
    float a2[32], a1[8], a3[2];
#pragma unroll
    for (int j = 0; j < 32; ++j) a2[j] = 0.0f;
#pragma unroll
    for (int j = 0; j < 8; ++j) a1[j] = 0.0f;
    a3[0] = a3[1] = 0.0f;
    float ab = 0.0f, ab3 = 0.0f, loss_local = 0.0f;
    const uint32_t o2 = tid >> 1, i2 = (tid & 1u) * 32u, i1 = (tid & 1u) * 8u, o3 = tid >> 5, i3 = (tid & 31u) * 2u;

    const uint32_t lane_addr = (warp * 32u) << 16;
    uint32_t phase = 0;
    const uint64_t tiles = (n + kRows - 1) / kRows;
    for (uint64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const uint64_t row = tile * kRows + tid;
        const bool live = row < n;
        uint4 f0 = make_uint4(0, 0, 0, 0), f1 = f0;
        if (live) {
            const uint4* src = reinterpret_cast<const uint4*>(feat + row * kIn);
            f0 = src[0];
            f1 = src[1];
        }
        *reinterpret_cast<uint4*>(s.x + core_off(tid, 0, kIn)) = f0;
        *reinterpret_cast<uint4*>(s.x + core_off(tid, 8, kIn)) = f1;
        operands_ready();
        // forward, keeping the ReLU masks of both hidden layers
        if (!tc_gemm(s.tc, 0, smem_addr(s.x), smem_addr(s.w1), kIn, 1, kIdescHid, phase)) break;
        float v[16];
        uint64_t m1 = 0, m2 = 0;
#pragma unroll 1
        for (uint32_t c0 = 0; c0 < kHid; c0 += 16) {
            tmem_ld16(s.tc.tmem + lane_addr + c0, v);
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                v[i] = fmaxf(v[i] + s.b1[c0 + i], 0.0f);
                if (v[i] > 0.0f) m1 |= 1ull << (c0 + i);
            }
            store_row16(s.h1, tid, c0, kHid, v);
        }
        operands_ready();
        if (!tc_gemm(s.tc, 64, smem_addr(s.h1), smem_addr(s.w2), kHid, 4, kIdescHid, phase)) break;
#pragma unroll 1
        for (uint32_t c0 = 0; c0 < kHid; c0 += 16) {
            tmem_ld16(s.tc.tmem + lane_addr + 64 + c0, v);
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                v[i] = fmaxf(v[i] + s.b2[c0 + i], 0.0f);
                if (v[i] > 0.0f) m2 |= 1ull << (c0 + i);
            }
            store_row16(s.h2, tid, c0, kHid, v);
        }
        operands_ready();
        if (!tc_gemm(s.tc, 0, smem_addr(s.h2), smem_addr(s.w3), kHid, 4, kIdescOut, phase)) break;
        // loss: sum of weight * (y - target)^2, times inv_norm
        tmem_ld16(s.tc.tmem + lane_addr, v);
        float dyv[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) dyv[i] = 0.0f;
        if (live) {
            const float4 t = target[row], w = weight[row];
            const float tt[4] = {t.x, t.y, t.z, t.w}, ww[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
            for (int o = 0; o < 4; ++o) {
                const float e = v[o] + s.b3[o] - tt[o];
                loss_local += ww[o] * e * e * inv_norm;
                dyv[o] = 2.0f * ww[o] * e * inv_norm;
            }
        }
#pragma unroll
        for (int o = 0; o < 4; ++o) s.dyf[tid * kOut + o] = dyv[o];
        store_row16(s.dy, tid, 0, kOutPad, dyv);
        operands_ready();
        // dH2 = dY W3 (into columns 64..127), dZ2 = dH2 * relu'(H2)
        if (!tc_gemm(s.tc, 64, smem_addr(s.dy), smem_addr(s.w3t), kOutPad, 1, kIdescHid, phase)) break;
#pragma unroll 1
        for (uint32_t c0 = 0; c0 < kHid; c0 += 16) {
            tmem_ld16(s.tc.tmem + lane_addr + 64 + c0, v);
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                v[i] = (m2 >> (c0 + i)) & 1ull ? v[i] : 0.0f;
                s.dz2f[tid * kHid + c0 + i] = v[i];
            }
            store_row16(s.dz2, tid, c0, kHid, v);
        }
        operands_ready();
        // dH1 = dZ2 W2 (into columns 0..63), dZ1 = dH1 * relu'(H1)
        if (!tc_gemm(s.tc, 0, smem_addr(s.dz2), smem_addr(s.w2t), kHid, 4, kIdescHid, phase)) break;
#pragma unroll 1
        for (uint32_t c0 = 0; c0 < kHid; c0 += 16) {
            tmem_ld16(s.tc.tmem + lane_addr + c0, v);
#pragma unroll
            for (int i = 0; i < 16; ++i) s.dz1f[tid * kHid + c0 + i] = (m1 >> (c0 + i)) & 1ull ? v[i] : 0.0f;
        }
        fence_before_sync();
        __syncthreads();
        // weight gradients over the tile's samples (CUDA cores)
#pragma unroll 1
        for (uint32_t t = 0; t < kRows; ++t) {
            const float g2 = s.dz2f[t * kHid + o2];
#pragma unroll
            for (uint32_t q = 0; q < 4; ++q) {
                const uint4 h = *reinterpret_cast<const uint4*>(s.h1 + core_off(t, i2 + q * 8, kHid));
                a2[q * 8 + 0] += g2 * bf16_lo(h.x);
                a2[q * 8 + 1] += g2 * bf16_hi(h.x);
                a2[q * 8 + 2] += g2 * bf16_lo(h.y);
                a2[q * 8 + 3] += g2 * bf16_hi(h.y);
                a2[q * 8 + 4] += g2 * bf16_lo(h.z);
                a2[q * 8 + 5] += g2 * bf16_hi(h.z);
                a2[q * 8 + 6] += g2 * bf16_lo(h.w);
                a2[q * 8 + 7] += g2 * bf16_hi(h.w);
            }
            const float g1 = s.dz1f[t * kHid + o2];
            const uint4 xv = *reinterpret_cast<const uint4*>(s.x + core_off(t, i1, kIn));
            a1[0] += g1 * bf16_lo(xv.x);
            a1[1] += g1 * bf16_hi(xv.x);
            a1[2] += g1 * bf16_lo(xv.y);
            a1[3] += g1 * bf16_hi(xv.y);
            a1[4] += g1 * bf16_lo(xv.z);
            a1[5] += g1 * bf16_hi(xv.z);
            a1[6] += g1 * bf16_lo(xv.w);
            a1[7] += g1 * bf16_hi(xv.w);
            const float g3 = s.dyf[t * kOut + o3];
            const uint32_t hv = *reinterpret_cast<const uint32_t*>(s.h2 + core_off(t, i3, kHid));
            a3[0] += g3 * bf16_lo(hv);
            a3[1] += g3 * bf16_hi(hv);
            ab += tid < kHid ? s.dz1f[t * kHid + tid] : s.dz2f[t * kHid + (tid - kHid)];
            if (tid < kOut) ab3 += s.dyf[t * kOut + tid];
        }
        __syncthreads();
    }
    const bool aborted = s.tc.abort != 0;
    tc_teardown(s.tc, phase, status, kTrainCols);
    if (aborted) return;
#pragma unroll
    for (int j = 0; j < 32; ++j) atomicAdd(grads + kOffW2 + o2 * kHid + i2 + j, a2[j]);
#pragma unroll
    for (int j = 0; j < 8; ++j) atomicAdd(grads + kOffW1 + o2 * kIn + i1 + j, a1[j]);
    atomicAdd(grads + kOffW3 + o3 * kHid + i3, a3[0]);
    atomicAdd(grads + kOffW3 + o3 * kHid + i3 + 1, a3[1]);
    atomicAdd(grads + (tid < kHid ? kOffB1 + tid : kOffB2 + tid - kHid), ab);
    if (tid < kOut) atomicAdd(grads + kOffB3 + tid, ab3);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) loss_local += __shfl_down_sync(0xffffffffu, loss_local, o);
    if ((tid & 31u) == 0) s.red[warp] = loss_local;
    __syncthreads();
    if (tid == 0) atomicAdd(loss, s.red[0] + s.red[1] + s.red[2] + s.red[3]);
}

// Adam on the FP32 parameters, then the BF16 copy the MMAs read.
__global__ void precond_adam_kernel(float* __restrict__ params, const float* __restrict__ grads,
                                    float* __restrict__ m, float* __restrict__ v, float lr, float b1, float b2,
                                    float eps, float bc1, float bc2, __nv_bfloat16* __restrict__ wbf) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= PDR_PRECOND_PARAMS) return;
    const float g = grads[i];
    const float mi = b1 * m[i] + (1.0f - b1) * g;
    const float vi = b2 * v[i] + (1.0f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    const float p = params[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    params[i] = p;
    wbf[i] = __float2bfloat16_rn(p);
}

// ---- per-texel statistics, features and the preconditioned update -----------------------------------

// One view: every masked pixel adds its bilinear tap weights to the texels' observation weight and
// marks them as seen by this view.
__global__ void observe_view_kernel(const float2* __restrict__ uv, const float* __restrict__ mask, uint64_t P,
                                    uint32_t tw, uint32_t th, float* __restrict__ obs, uint8_t* __restrict__ seen) {
    const uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P || !(mask[p] > 0.0f)) return;
    const float2 u = uv[p];
    const float px = u.x * (float)tw - 0.5f, py = u.y * (float)th - 0.5f;
    const int32_t bx = f2i_sat(floorf(px)), by = f2i_sat(floorf(py));
    const float fx = px - floorf(px), fy = py - floorf(py);
    const uint32_t x0 = (uint32_t)clampi(bx, 0, (int32_t)tw - 1), x1 = (uint32_t)clampi(add1(bx), 0, (int32_t)tw - 1);
    const uint32_t y0 = (uint32_t)clampi(by, 0, (int32_t)th - 1), y1 = (uint32_t)clampi(add1(by), 0, (int32_t)th - 1);
    const float m = mask[p];
    const uint32_t o[4] = {y0 * tw + x0, y0 * tw + x1, y1 * tw + x0, y1 * tw + x1};
    const float w[4] = {(1.0f - fx) * (1.0f - fy), fx * (1.0f - fy), (1.0f - fx) * fy, fx * fy};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (w[k] > 0.0f) {
            atomicAdd(obs + o[k], w[k] * m);
            seen[o[k]] = 1;
        }
    }
}

__global__ void count_views_kernel(uint8_t* __restrict__ seen, float* __restrict__ views, uint64_t N) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    if (seen[i]) {
        views[i] += 1.0f;
        seen[i] = 0;
    }
}

// Distance proxy to the nearest chart edge: the smallest r in {1, 2, 4, ..., 32} for which one of the
// eight texels at offset r lies outside the atlas, is invalid or belongs to another chart (64 when none).
__global__ void edge_distance_kernel(const uint8_t* __restrict__ valid, const int32_t* __restrict__ chart,
                                     uint32_t tw, uint32_t th, float* __restrict__ edge) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= tw * th) return;
    const int32_t x = (int32_t)(i % tw), y = (int32_t)(i / tw);
    const int32_t c = chart ? chart[i] : 0;
    float d = 64.0f;
    if (!valid[i]) {
        d = 0.0f;
    } else {
        for (int32_t r = 1; r <= 32 && d == 64.0f; r <<= 1) {
            const int32_t dx[8] = {r, -r, 0, 0, r, r, -r, -r}, dy[8] = {0, 0, r, -r, r, -r, r, -r};
            for (int k = 0; k < 8; ++k) {
                const int32_t xx = x + dx[k], yy = y + dy[k];
                bool edge_hit = xx < 0 || yy < 0 || xx >= (int32_t)tw || yy >= (int32_t)th;
                if (!edge_hit) {
                    const uint32_t j = (uint32_t)yy * tw + (uint32_t)xx;
                    edge_hit = !valid[j] || (chart && chart[j] != c);
                }
                if (edge_hit) {
                    d = (float)r;
                    break;
                }
            }
        }
    }
    edge[i] = d;
}

__device__ __forceinline__ float signed_log(float x) {
    const float a = fabsf(x);
    const float l = a > 1e-12f ? (log10f(a) + 12.0f) / 12.0f : 0.0f;
    return x < 0.0f ? -l : l;
}

// Per-texel features (BF16 [N][16]) from the refine state:
//   0-2   Adam direction m^ / (sqrt(v^) + eps) per channel, clamped to +-4
//   3-5   signed log10 magnitude of m^, (log10|m^| + 12) / 12
//   6-8   log10 magnitude of sqrt(v^), same scale
//   9-11  texel value - 0.5
//   12    log(1 + observation weight) / 8
//   13    views that see the texel / 16
//   14    chart-edge distance proxy / 64
//   15    fraction of the schedule done
__global__ void features_kernel(const float* __restrict__ tex, const float* __restrict__ m1,
                                const float* __restrict__ m2, float bc1, float bc2, float eps,
                                const float* __restrict__ obs, const float* __restrict__ views,
                                const float* __restrict__ edge, float progress, uint64_t N,
                                __nv_bfloat16* __restrict__ feat) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    float f[16];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float mh = m1[i * 3 + c] / bc1, vh = sqrtf(m2[i * 3 + c] / bc2);
        f[c] = fminf(fmaxf(mh / (vh + eps), -4.0f), 4.0f);
        f[3 + c] = signed_log(mh);
        f[6 + c] = signed_log(vh);
        f[9 + c] = tex[i * 3 + c] - 0.5f;
    }
    f[12] = logf(1.0f + obs[i]) * 0.125f;
    f[13] = views[i] * 0.0625f;
    f[14] = edge[i] * (1.0f / 64.0f);
    f[15] = progress;
    uint4 a, b;
    a.x = pack_bf16(f[0], f[1]);
    a.y = pack_bf16(f[2], f[3]);
    a.z = pack_bf16(f[4], f[5]);
    a.w = pack_bf16(f[6], f[7]);
    b.x = pack_bf16(f[8], f[9]);
    b.y = pack_bf16(f[10], f[11]);
    b.z = pack_bf16(f[12], f[13]);
    b.w = pack_bf16(f[14], f[15]);
    uint4* dst = reinterpret_cast<uint4*>(feat + i * kIn);
    dst[0] = a;
    dst[1] = b;
}

// Adam with a per-texel, per-channel step multiplier exp(clamp(out_c, log 1/8, log 16)); the
// multipliers are ignored (plain Adam) once *fallback is set. Arithmetic as adam_kernel, streamed the
// same way (four consecutive values per thread; value k belongs to texel k / 3, channel k % 3).
__device__ __forceinline__ void adam_scaled_one(float& x, float& g, float& m, float& v, float s, float lr, float b1,
                                                float b2, float eps, float bc1, float bc2, float cmin, float cmax) {
    const float mm = b1 * m + (1.0f - b1) * g;
    const float vv = b2 * v + (1.0f - b2) * g * g;
    m = mm;
    v = vv;
    x = clamp_hlsl(x - lr * s * (mm / bc1) / (sqrtf(vv / bc2) + eps), cmin, cmax);
    g = 0.0f;
}

__device__ __forceinline__ float step_multiplier(const float* __restrict__ mult, uint64_t k, bool plain) {
    if (plain) return 1.0f;
    const uint64_t t = k / 3;
    return expf(fminf(fmaxf(mult[t * 4 + (k - t * 3)], -2.0794415f), 2.7725887f));
}

__global__ void __launch_bounds__(256, 8)  // 32 registers: full occupancy for the streaming update
adam_scaled_kernel(float* __restrict__ tex, float* __restrict__ grad, float* __restrict__ m1,
                                   float* __restrict__ m2, uint64_t texels, const float* __restrict__ mult,
                                   const uint32_t* __restrict__ fallback, float lr, float b1, float b2, float eps,
                                   float bc1, float bc2, float cmin, float cmax) {
    // one texel per thread, as adam_kernel: texture and moments [texels][3], gradient and multipliers
    // [texels][4]
    const bool plain = *fallback != 0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < texels; t += stride) {
        const float4 d = reinterpret_cast<const float4*>(grad)[t];
        float g[3] = {d.x, d.y, d.z};
#pragma unroll
        for (int c = 0; c < 3; ++c)
            adam_scaled_one(tex[t * 3 + c], g[c], m1[t * 3 + c], m2[t * 3 + c], step_multiplier(mult, t * 3 + c, plain),
                            lr, b1, b2, eps, bc1, bc2, cmin, cmax);
        reinterpret_cast<float4*>(grad)[t] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
}

// Plain-Adam fallback: after each refresh window, if the mean batch loss of the last window rose by more
// than `tolerance` over the window before, the multipliers are switched off for the rest of the run.
__global__ void fallback_check_kernel(const float* __restrict__ loss, uint32_t begin, uint32_t window, float tolerance,
                                      uint32_t* __restrict__ fallback) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    float prev = 0.0f, last = 0.0f;
    for (uint32_t k = 0; k < window; ++k) {
        prev += loss[begin + k];
        last += loss[begin + window + k];
    }
    if (last > prev * (1.0f + tolerance)) *fallback = 1u;
}

template <class F>
cudaError_t set_smem(F* kernel, size_t bytes) {
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

uint32_t grid_for(uint64_t tiles, uint32_t per_sm) {
    const uint64_t cap = (uint64_t)num_sms() * per_sm;
    return (uint32_t)(tiles < cap ? (tiles ? tiles : 1) : cap);
}

}  // namespace

// Resident forward CTAs per SM: 4 x (33 KB shared memory, 128 threads x 94 registers, 64 TMEM columns) fits
// every limit of an SM (228 KB, 64K registers, 512 TMEM columns) with room to spare.
constexpr uint32_t kForwardCtasPerSm = 4;

cudaError_t precond_prepare() {
    static const cudaError_t fwd = [] {
        const cudaError_t e = set_smem(precond_forward_kernel, sizeof(FwdSmem));
        if (e != cudaSuccess) return e;
        return cudaFuncSetAttribute(precond_forward_kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                    (int)cudaSharedmemCarveoutMaxShared);
    }();
    static const cudaError_t train = set_smem(precond_train_kernel, sizeof(TrainSmem));
    return fwd != cudaSuccess ? fwd : train;
}

cudaError_t launch_precond_forward(const float* params, const uint16_t* wbf, const uint16_t* feat, uint64_t n,
                                   float* out, uint32_t* status, cudaStream_t stream) {
    const cudaError_t attr = precond_prepare();
    if (attr != cudaSuccess) return attr;
    const uint64_t tiles = (n + kRows - 1) / kRows;
    precond_forward_kernel<<<grid_for(tiles, kForwardCtasPerSm), kThreads, sizeof(FwdSmem), stream>>>(
        params, reinterpret_cast<const __nv_bfloat16*>(wbf), reinterpret_cast<const __nv_bfloat16*>(feat), n,
        reinterpret_cast<float4*>(out), status);
    return cudaGetLastError();
}

cudaError_t launch_precond_train(const float* params, const uint16_t* wbf, const uint16_t* feat, const float* target,
                                 const float* weight, uint64_t n, float inv_norm, float* grads, float* loss,
                                 uint32_t* status, cudaStream_t stream) {
    const cudaError_t attr = precond_prepare();
    if (attr != cudaSuccess) return attr;
    cudaError_t err = cudaMemsetAsync(grads, 0, PDR_PRECOND_PARAMS * sizeof(float), stream);
    if (err == cudaSuccess) err = cudaMemsetAsync(loss, 0, sizeof(float), stream);
    if (err != cudaSuccess) return err;
    const uint64_t tiles = (n + kRows - 1) / kRows;
    precond_train_kernel<<<grid_for(tiles, 1), kThreads, sizeof(TrainSmem), stream>>>(
        params, reinterpret_cast<const __nv_bfloat16*>(wbf), reinterpret_cast<const __nv_bfloat16*>(feat),
        reinterpret_cast<const float4*>(target), reinterpret_cast<const float4*>(weight), n, inv_norm, grads, loss,
        status);
    return cudaGetLastError();
}

cudaError_t launch_precond_adam(float* params, const float* grads, float* m, float* v, float lr, float b1, float b2,
                                float eps, float bc1, float bc2, uint16_t* wbf, cudaStream_t stream) {
    precond_adam_kernel<<<(PDR_PRECOND_PARAMS + 255) / 256, 256, 0, stream>>>(
        params, grads, m, v, lr, b1, b2, eps, bc1, bc2, reinterpret_cast<__nv_bfloat16*>(wbf));
    return cudaGetLastError();
}

cudaError_t launch_observe_view(const float* uv, const float* mask, uint64_t P, uint32_t tw, uint32_t th, float* obs,
                                uint8_t* seen, float* views, cudaStream_t stream) {
    observe_view_kernel<<<(unsigned)((P + 255) / 256), 256, 0, stream>>>(reinterpret_cast<const float2*>(uv), mask, P,
                                                                         tw, th, obs, seen);
    const uint64_t N = (uint64_t)tw * th;
    count_views_kernel<<<(unsigned)((N + 255) / 256), 256, 0, stream>>>(seen, views, N);
    return cudaGetLastError();
}

cudaError_t launch_edge_distance(const uint8_t* valid, const int32_t* chart, uint32_t tw, uint32_t th, float* edge,
                                 cudaStream_t stream) {
    edge_distance_kernel<<<(tw * th + 255) / 256, 256, 0, stream>>>(valid, chart, tw, th, edge);
    return cudaGetLastError();
}

cudaError_t launch_precond_features(const float* tex, const float* m1, const float* m2, float bc1, float bc2,
                                    float eps, const float* obs, const float* views, const float* edge, float progress,
                                    uint64_t N, uint16_t* feat, cudaStream_t stream) {
    features_kernel<<<(unsigned)((N + 255) / 256), 256, 0, stream>>>(tex, m1, m2, bc1, bc2, eps, obs, views, edge,
                                                                     progress, N,
                                                                     reinterpret_cast<__nv_bfloat16*>(feat));
    return cudaGetLastError();
}

cudaError_t launch_adam_scaled(float* tex, float* grad, float* m1, float* m2, uint64_t N, const float* mult,
                               const uint32_t* fallback, float lr, float b1, float b2, float eps, float bc1, float bc2,
                               float cmin, float cmax, cudaStream_t stream) {
    uint64_t blocks = (N + 255) / 256;  // one texel per thread, as launch_adam
    if (blocks > 0x7FFFFFFFu) blocks = 0x7FFFFFFFu;
    if (blocks == 0) blocks = 1;
    adam_scaled_kernel<<<(unsigned)blocks, 256, 0, stream>>>(tex, grad, m1, m2, N, mult, fallback, lr, b1, b2, eps,
                                                             bc1, bc2, cmin, cmax);
    return cudaGetLastError();
}

cudaError_t launch_fallback_check(const float* loss, uint32_t begin, uint32_t window, float tolerance,
                                  uint32_t* fallback, cudaStream_t stream) {
    fallback_check_kernel<<<1, 32, 0, stream>>>(loss, begin, window, tolerance, fallback);
    return cudaGetLastError();
}

}  // namespace pdr
