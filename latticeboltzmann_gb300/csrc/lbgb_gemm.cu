// BF16 GEMM with FP32 accumulation for the Fourier-neural-operator layers:
//   C = alpha * A * B + beta * C,  A (m x k), B (k x n) in BF16, C FP32,
// every operand addressed by (row stride, column stride) and a batch stride,
// so row-major, column-major and transposed views all go through one call.
//
// Tensor-core path (k_gemm_tc): one CTA of 128 threads computes a 128 x NT
// tile of C with tcgen05.mma (kind::f16, BF16 inputs, FP32 accumulator held
// in tensor memory).  Per 64-wide K block the threads copy A (128 x 64) and B
// (NT x 64) into shared memory in the canonical K-major layout without
// swizzle -- 8x8 "core matrices" of 16-byte rows, neighbours along K 128 B
// apart (leading byte offset), neighbours along M/N 1024 B apart (stride byte
// offset) -- one elected thread issues four K=16 MMAs and commits them to an
// mbarrier, and all threads wait (bounded) before reusing the buffers.  The
// epilogue reads the accumulator rows back with tcgen05.ld (warp w owns TMEM
// lanes 32w..32w+31) and applies alpha/beta.
//
// SIMT path (k_gemm_simt): the same contract with FP32 FMAs; the reference the
// tensor-core path is tested against.
#include <cuda.h>
#include <stdio.h>

#include <type_traits>

#include "lbgb_act.cuh"
#include "lbgb_common.cuh"

namespace lbgb {

__device__ int g_gemm_status;

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor (tcgen05): start address, leading and stride
// byte offsets (16-byte units), descriptor version bit 46, layout type in
// bits 61-63 (0: no swizzle, 2: 128-byte swizzle)
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo, uint32_t layout = 0) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3ffffu) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3fffu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3fffu) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)(layout & 7u) << 61;
    return d;
}

// instruction descriptor for kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N and M encoded as N/8 and M/16
__host__ __device__ constexpr uint32_t umma_idesc_bf16(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void mbar_init_g(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait_g(uint64_t *bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return done != 0;
}
__device__ __forceinline__ bool mbar_wait_g(uint64_t *bar, uint32_t parity, long long limit) {
    for (long long i = 0; i < limit; ++i)
        if (mbar_try_wait_g(bar, parity)) return true;
    return false;
}

__device__ __forceinline__ void store_out(float *p, float x) { *p = x; }
__device__ __forceinline__ void store_out(__nv_bfloat16 *p, float x) { *p = __float2bfloat16_rn(x); }
__device__ __forceinline__ float load_out(const float *p) { return *p; }
__device__ __forceinline__ float load_out(const __nv_bfloat16 *p) { return __bfloat162float(*p); }
// four consecutive outputs (16 bytes of FP32, 8 of BF16; aligned)
__device__ __forceinline__ void load4_out(const float *p, float (&x)[4]) {
    const float4 v = *reinterpret_cast<const float4 *>(p);
    x[0] = v.x, x[1] = v.y, x[2] = v.z, x[3] = v.w;
}
__device__ __forceinline__ void load4_out(const __nv_bfloat16 *p, float (&x)[4]) {
    const uint2 v = *reinterpret_cast<const uint2 *>(p);
    x[0] = __uint_as_float(v.x << 16), x[1] = __uint_as_float(v.x & 0xffff0000u);
    x[2] = __uint_as_float(v.y << 16), x[3] = __uint_as_float(v.y & 0xffff0000u);
}
__device__ __forceinline__ uint2 pack4_bf16(const float (&x)[4]) {
    const uint32_t a = (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(x[0])) |
                       ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(x[1])) << 16);
    const uint32_t b = (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(x[2])) |
                       ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(x[3])) << 16);
    return make_uint2(a, b);
}
__device__ __forceinline__ void store4_out(float *p, const float (&x)[4]) {
    *reinterpret_cast<float4 *>(p) = make_float4(x[0], x[1], x[2], x[3]);
}
__device__ __forceinline__ void store4_out(__nv_bfloat16 *p, const float (&x)[4]) {
    *reinterpret_cast<uint2 *>(p) = pack4_bf16(x);
}

constexpr int TC_M = 128;
constexpr long long TC_WAIT = 1ll << 22;

// Copies rows [r0, r0+ROWS) x k [k0, k0+64) of X (element (r, k) at
// X[r * rs + k * ks], zero outside R x K) into the core-matrix K-major layout.
// Thread-to-element mapping follows the contiguous axis so that a warp's
// loads coalesce: 16-byte vector loads along K when K is contiguous and
// aligned, consecutive rows per warp when the rows are contiguous.  Every
// thread moves exactly ITERS 16-byte pieces (the tile sizes are multiples of
// 128 pieces): all its loads are issued before the first shared-memory store,
// so their DRAM latencies overlap instead of adding up.
// zero_rows: write the zeros of rows past R too; a stage whose zero rows were
// written by an earlier K block still holds them (they never change).
template <int ROWS, int KB>
__device__ __forceinline__ void load_tile(unsigned char *dst, const __nv_bfloat16 *__restrict__ X, long long rs,
                                          long long ks, int r0, int R, int k0, int K, int tid,
                                          unsigned short *stage, bool zero_rows) {
    constexpr int ITERS = ROWS * KB / 8 / 128;
    static_assert(ITERS >= 1 && ROWS * KB / 8 == ITERS * 128, "tile of whole 128-piece rounds");
    const bool row_contig = rs == 1 && ks != 1;
    if (row_contig && (ks & 7) == 0 && r0 + ROWS <= R && (reinterpret_cast<uintptr_t>(X) & 15) == 0) {
        // rows contiguous (an M- or N-major operand): 16-byte loads of 8 rows
        // at one k into a [k][row] staging tile, then each thread gathers the
        // 8 k values of one row into a 16-byte core-matrix row
        constexpr int G = ROWS / 8;
        uint4 w[ITERS];
#pragma unroll
        for (int it = 0; it < ITERS; ++it) {
            const int e = tid + it * 128;
            const int kk = e / G, g = e - kk * G;
            const int gk = k0 + kk;
            w[it] = make_uint4(0u, 0u, 0u, 0u);
            if (gk < K)
                w[it] = __ldg(reinterpret_cast<const uint4 *>(X + (long long)(r0 + 8 * g) + (long long)gk * ks));
        }
#pragma unroll
        for (int it = 0; it < ITERS; ++it) {
            const int e = tid + it * 128;
            const int kk = e / G, g = e - kk * G;
            *reinterpret_cast<uint4 *>(stage + kk * ROWS + 8 * g) = w[it];
        }
        __syncthreads();
        for (int e = tid; e < ROWS * (KB / 8); e += 128) {
            const int r = e % ROWS, kc = e / ROWS;
            unsigned short h[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) h[q] = stage[(kc * 8 + q) * ROWS + r];
            uint4 w;
            memcpy(&w, h, 16);
            *reinterpret_cast<uint4 *>(dst + (r >> 3) * (KB * 16) + kc * 128 + (r & 7) * 16) = w;
        }
        __syncthreads();  // the staging tile is reused by the next operand
        return;
    }
    const bool vec = ks == 1 && (rs & 7) == 0 && ((reinterpret_cast<uintptr_t>(X) & 15) == 0);
    if (vec && k0 + KB <= K) {
        // K contiguous and the whole K block inside X: 16-byte loads only
        // (rows past R are zeros)
        uint4 w[ITERS];
#pragma unroll
        for (int it = 0; it < ITERS; ++it) {
            const int e = tid + it * 128, r = e / (KB / 8), kc = e % (KB / 8);
            w[it] = make_uint4(0u, 0u, 0u, 0u);
            if (r0 + r < R) w[it] = __ldg(reinterpret_cast<const uint4 *>(X + (long long)(r0 + r) * rs + (k0 + kc * 8)));
        }
#pragma unroll
        for (int it = 0; it < ITERS; ++it) {
            const int e = tid + it * 128, r = e / (KB / 8), kc = e % (KB / 8);
            if (zero_rows || r0 + r < R)
                *reinterpret_cast<uint4 *>(dst + (r >> 3) * (KB * 16) + kc * 128 + (r & 7) * 16) = w[it];
        }
        return;
    }
    for (int e = tid; e < ROWS * KB / 8; e += 128) {
        int r, kc;
        if (row_contig) {
            r = e % ROWS;
            kc = e / ROWS;
        } else {
            r = e / (KB / 8);
            kc = e % (KB / 8);
        }
        const int gr = r0 + r, gk = k0 + kc * 8;
        uint4 w = make_uint4(0u, 0u, 0u, 0u);
        if (gr < R) {
            const __nv_bfloat16 *p = X + (long long)gr * rs + (long long)gk * ks;
            if (vec && gk + 8 <= K) {
                w = __ldg(reinterpret_cast<const uint4 *>(p));
            } else {
                unsigned short h[8];
#pragma unroll
                for (int q = 0; q < 8; ++q) h[q] = gk + q < K ? __bfloat16_as_ushort(p[(long long)q * ks]) : 0;
                memcpy(&w, h, 16);
            }
        }
        *reinterpret_cast<uint4 *>(dst + (r >> 3) * (KB * 16) + kc * 128 + (r & 7) * 16) = w;
    }
}

// Bytes of dynamic shared memory a variant needs: its operand stages (A then
// B, each stage 1024-byte aligned) and the staging area (a [k][row] tile of a
// row-contiguous operand, or the epilogue's 4 x 32 x 17 floats).
template <int NT, int KB, int ST>
__host__ __device__ constexpr int tc_operand_bytes() { return ST * (TC_M + NT) * KB * 2; }
template <int KB>
__host__ __device__ constexpr int tc_stage_bytes() { return KB * TC_M * 2 > 8704 ? KB * TC_M * 2 : 8704; }

template <int NT, typename OUT, int KB, int ST>
__global__ void __launch_bounds__(128, 1)
k_gemm_tc(int M, int N, int K, const __nv_bfloat16 *__restrict__ A, long long a_rs, long long a_cs, long long a_bs,
          const __nv_bfloat16 *__restrict__ B, long long b_rs, long long b_cs, long long b_bs, OUT *__restrict__ C,
          long long c_rs, long long c_cs, long long c_bs, float alpha, float beta) {
    static_assert(NT % 16 == 0 && NT >= 32 && NT <= 256, "tile N");
    static_assert(KB == 32 || KB == 64, "K block");
    static_assert(ST == 1 || ST == 2, "stages");
    constexpr int A_BYTES = TC_M * KB * 2, B_BYTES = NT * KB * 2;
    // dynamic shared memory: ST stages of A, ST stages of B, then the staging
    // area of row-contiguous operands and of row-major output
    extern __shared__ __align__(1024) unsigned char dsm[];
    unsigned char *sA0 = dsm;
    unsigned char *sB0 = dsm + ST * A_BYTES;
    unsigned short *stage = reinterpret_cast<unsigned short *>(dsm + tc_operand_bytes<NT, KB, ST>());
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ uint32_t tmem_slot;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * TC_M, n0 = blockIdx.y * NT;
    const long long z = blockIdx.z;
    A += z * a_bs;
    B += z * b_bs;
    C += z * c_bs;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "r"((uint32_t)NT)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        mbar_init_g(&bar[0], 1);
        mbar_init_g(&bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;
    constexpr uint32_t idesc = umma_idesc_bf16(TC_M, NT);

    // K blocks: block kb is staged in stage kb % ST and its MMAs commit to
    // bar[kb % 2]; with two stages the loads of block kb overlap the MMAs of
    // block kb-1, and a stage is refilled only after the MMAs of block kb-2
    // (which read it) have completed.  Commits complete in order, so the last
    // one completing means every MMA has.
    bool ok = true;
    int issued = -1;
    const int kblocks = (K + KB - 1) / KB;
    for (int kb = 0; kb < kblocks; ++kb) {
        const int st = ST == 2 ? (kb & 1) : 0;
        if (kb >= ST) {
            const int prev = kb - ST;  // the block whose MMAs read this stage last
            const bool w = mbar_wait_g(&bar[prev & 1], (uint32_t)(prev >> 1) & 1u, TC_WAIT);
            if (!w) atomicCAS(&g_gemm_status, 0, 1);
            ok = __syncthreads_and(w) != 0;  // every thread leaves together if a wait gave up
            if (!ok) break;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        }
        const int k0 = kb * KB;
        unsigned char *sA = sA0 + st * A_BYTES, *sB = sB0 + st * B_BYTES;
        // A tile: 128 rows x KB k; element (r, kk) at (r/8)*KB*16 + (kk/8)*128 + (r%8)*16 + (kk%8)*2
        load_tile<TC_M, KB>(sA, A, a_rs, a_cs, m0, M, k0, K, tid, stage, kb < ST);
        // B tile: NT rows (n) x KB k, same layout; B(k, n) = B[k * b_rs + n * b_cs]
        load_tile<NT, KB>(sB, B, b_cs, b_rs, n0, N, k0, K, tid, stage, kb < ST);
        // make the generic-proxy writes visible to the tensor core
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
            for (int kk = 0; kk < KB / 16; ++kk) {
                // K = 16 per MMA: two core matrices along K, 256 bytes
                const uint64_t da = umma_desc(smem_u32(sA) + kk * 256, 128, KB * 16);
                const uint64_t db = umma_desc(smem_u32(sB) + kk * 256, 128, KB * 16);
                const uint32_t acc = (kb > 0 || kk > 0) ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\t"
                    "setp.ne.u32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
                    "l"(da), "l"(db), "r"(idesc), "r"(acc)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(&bar[kb & 1]))
                         : "memory");
        }
        issued = kb;
    }
    if (issued >= 0) {
        // the last block's MMAs (bounded; on a timeout wait once more before
        // the buffers and the tensor memory go away)
        const bool w = mbar_wait_g(&bar[issued & 1], (uint32_t)(issued >> 1) & 1u, TC_WAIT);
        if (!w) {
            atomicCAS(&g_gemm_status, 0, 1);
            mbar_wait_g(&bar[issued & 1], (uint32_t)(issued >> 1) & 1u, TC_WAIT);
        }
        ok = __syncthreads_and(ok && w) != 0;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    } else {
        ok = false;  // K = 0 is handled on the host; nothing to read back
    }

    if (ok && c_cs == 1 && c_rs != 1) {
        // row-major C: each warp stages its 32 x 16 block in shared memory (the
        // dynamic staging area; a 17-float pitch keeps the banks distinct) and
        // writes it two rows per instruction, 16 consecutive columns each, so
        // the stores coalesce instead of 32 lanes hitting 32 rows
        float *ostage = reinterpret_cast<float *>(stage) + warp * (32 * 17);
#pragma unroll 1
        for (int c0 = 0; c0 < NT; c0 += 16) {
            uint32_t v[16];
            const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
                "%14, %15}, [%16];"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                  "=r"(v[15])
                : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (int j = 0; j < 16; ++j) ostage[lane * 17 + j] = __uint_as_float(v[j]);
            __syncwarp();
            // the 16 old values of C (beta != 0) are all requested before any
            // is used, so their latencies overlap
            const int j = lane & 15, col = n0 + c0 + j;
            float old[16];
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                const int row = m0 + warp * 32 + 2 * i + (lane >> 4);
                old[i] = (beta != 0.f && row < M && col < N) ? load_out(C + (long long)row * c_rs + col) : 0.f;
            }
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                const int r = 2 * i + (lane >> 4);
                const int row = m0 + warp * 32 + r;
                if (row < M && col < N)
                    store_out(C + (long long)row * c_rs + col, alpha * ostage[r * 17 + j] + beta * old[i]);
            }
            __syncwarp();
        }
    } else if (ok) {
        // epilogue: warp w reads TMEM lanes 32w..32w+31 = rows m0+32w+lane
        const int row = m0 + warp * 32 + lane;
#pragma unroll 1
        for (int c0 = 0; c0 < NT; c0 += 16) {
            uint32_t v[16];
            const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
                "%14, %15}, [%16];"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                  "=r"(v[15])
                : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (row < M) {
                float old[16];
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int col = n0 + c0 + j;
                    old[j] = (beta != 0.f && col < N) ? load_out(C + (long long)row * c_rs + (long long)col * c_cs)
                                                      : 0.f;
                }
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int col = n0 + c0 + j;
                    if (col < N)
                        store_out(C + (long long)row * c_rs + (long long)col * c_cs,
                                  alpha * __uint_as_float(v[j]) + beta * old[j]);
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)NT)
                     : "memory");
}

// SIMT reference: 16x16 threads, 64x64 tile, FP32 accumulation
template <typename OUT>
__global__ void __launch_bounds__(256)
k_gemm_simt(int M, int N, int K, const __nv_bfloat16 *__restrict__ A, long long a_rs, long long a_cs, long long a_bs,
            const __nv_bfloat16 *__restrict__ B, long long b_rs, long long b_cs, long long b_bs, OUT *__restrict__ C,
            long long c_rs, long long c_cs, long long c_bs, float alpha, float beta) {
    __shared__ float As[16][65];
    __shared__ float Bs[16][65];
    const long long z = blockIdx.z;
    A += z * a_bs;
    B += z * b_bs;
    C += z * c_bs;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int m0 = blockIdx.x * 64, n0 = blockIdx.y * 64;
    float acc[4][4] = {};
    for (int k0 = 0; k0 < K; k0 += 16) {
        for (int e = threadIdx.x; e < 16 * 64; e += 256) {
            const int kk = e >> 6, i = e & 63;
            const int gm = m0 + i, gn = n0 + i, gk = k0 + kk;
            As[kk][i] = (gm < M && gk < K) ? __bfloat162float(A[(long long)gm * a_rs + (long long)gk * a_cs]) : 0.f;
            Bs[kk][i] = (gn < N && gk < K) ? __bfloat162float(B[(long long)gk * b_rs + (long long)gn * b_cs]) : 0.f;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 16; ++kk)
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) acc[a][b] += As[kk][ty * 4 + a] * Bs[kk][tx * 4 + b];
        __syncthreads();
    }
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int gm = m0 + ty * 4 + a, gn = n0 + tx * 4 + b;
            if (gm < M && gn < N) {
                OUT *cp = C + (long long)gm * c_rs + (long long)gn * c_cs;
                store_out(cp, beta == 0.f ? alpha * acc[a][b] : alpha * acc[a][b] + beta * load_out(cp));
            }
        }
}

// Dynamic shared memory of one tensor-core GEMM variant: the staging area
// (a [k][row] tile, or the epilogue's 4 x 32 x 17 floats), grown until the
// CTAs that fit on one SM hold at most the SM's 512 tensor-memory columns, so
// that no allocation ever waits.  Computed once per variant and device.
template <int NT, typename OUT, int KB, int ST>
static int tc_dyn_smem() {
    static std::atomic<int> cache[MAX_DEVICES];
    const int dev = current_device();
    const int have = cache[dev].load(std::memory_order_acquire);
    if (have) return have;
    std::lock_guard<std::mutex> lock(setup_mutex());
    int d = tc_operand_bytes<NT, KB, ST>() + tc_stage_bytes<KB>();
    for (;;) {
        cudaFuncSetAttribute(k_gemm_tc<NT, OUT, KB, ST>, cudaFuncAttributeMaxDynamicSharedMemorySize, d);
        int nb = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_gemm_tc<NT, OUT, KB, ST>, 128, d) != cudaSuccess)
            break;
        if (nb * NT <= 512 || d >= 200 * 1024) break;
        d += 1024;
    }
    cache[dev].store(d, std::memory_order_release);
    return d;
}

// ---------------------------------------------------------------- TMA pipeline
// Persistent, warp-specialised GEMM for products whose B is K-major
// (B(k, n) = B[n * b_cs + k]) and whose A is K-major (A(r, k) = A[r * a_rs + k])
// or M-major (A(r, k) = A[k * a_cs + r]), rows 16-byte aligned -- the
// forward W and H transforms, the inverse W transform, the split-K weight
// gradients and the forward pointwise layers and projections of the
// surrogate.
//
//  * warp 0, one thread: TMA producer.  Per 64-deep K block it issues one
//    cp.async.bulk.tensor load of A (128 rows x 64 k) and one of B (NT rows
//    x 64 k): 128-byte rows with the 128-byte swizzle, which is the
//    tcgen05 K-major SWIZZLE_128B layout (8-row atoms of 1024 bytes; the
//    MMAs step through K by advancing the descriptor 32 bytes).
//    Out-of-range rows and k read as zeros.  A ring of STAGES stages,
//    full/empty mbarriers.
//  * warp 1, one thread: issues tcgen05.mma (M = 128, N = NT, K = 16) into
//    one of two TMEM accumulators and commits each stage back to the
//    producer and each finished tile to the epilogue.
//  * warps 2-9: epilogue.  Warp w reads TMEM lanes 32 (w % 4) .. + 31 (the
//    lane quarter it may access) and half of the tile's columns, applies
//    alpha/beta and stores; then frees the accumulator, so the MMAs of the
//    next tile run while this one drains.
// Every wait is bounded: a timeout sets the status word and ends that role's
// loop; the other roles' bounded waits then run out in turn, the producer
// waits for its copies in flight and the MMA thread for its last commit
// before the tensor memory is released.
constexpr int TP_KB = 64;
constexpr int TP_THREADS = 320;

template <int NT>
struct TmaShape {
    static constexpr int A_BYTES = TC_M * TP_KB * 2;
    static constexpr int B_BYTES = NT * TP_KB * 2;
    static constexpr int STAGE = A_BYTES + B_BYTES;
    // two CTAs per SM: ~82-97 KB of dynamic shared memory each
    static constexpr int STAGES = NT == 128 ? 2 : (NT == 64 ? 3 : 4);
    static constexpr int EPI = 8 * 32 * 17 * 4;
    static constexpr int SMEM = STAGES * STAGE + EPI;
};

__device__ __forceinline__ void mbar_arrive_g(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx_g(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// one box of a 2-D (x = k, y = row) or 3-D (z = problem) tensor map
__device__ __forceinline__ void tma_load_box(void *dst, const CUtensorMap *map, bool three_d, int x, int y, int z,
                                             uint64_t *bar) {
    if (three_d)
        asm volatile(
            "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
            "[%5];" ::"r"(smem_u32(dst)),
            "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
            : "memory");
    else
        asm volatile(
            "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
                smem_u32(dst)),
            "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
            : "memory");
}
__device__ __forceinline__ void tc_ld16(uint32_t taddr, uint32_t (&v)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
        "%14, %15}, [%16];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
          "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Optional epilogue of a surrogate layer, applied by the TMA pipeline to a
// row-major FP32 C of one problem: C += bias[row / rows] after alpha/beta,
// and vb = BF16(act ? GELU(C) : C) at the same offset -- what lbgb_fno_bias_act
// does as a separate pass over C.
struct Epi {
    const float *bias = nullptr;
    long long rows = 1;
    int act = 0;
    __nv_bfloat16 *vb = nullptr;
};

// AMN: A is M-major (m contiguous, A(m, k) = A[k * a_cs + m]; the
// channel-major activations of the pointwise layers).  Its tile is then two
// 64-element-wide boxes per K block (m0 and m0 + 64), each 64 k rows of 128
// bytes with the 128-byte swizzle: the MN-major SWIZZLE_128B layout, 8-row
// K groups 1024 bytes apart, the two 64-element M chunks 8192 bytes apart;
// an MMA of K = 16 starts 2048 bytes further.
template <int NT, typename OUT, bool AMN = false, bool EPI = false>
__global__ void __launch_bounds__(TP_THREADS, 2)
k_gemm_tma(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int a3d, int b3d, int M,
           int N, int K, int batch, OUT *__restrict__ C, long long c_rs, long long c_cs, long long c_bs, float alpha,
           float beta, Epi ep) {
    using S = TmaShape<NT>;
    constexpr int STAGES = S::STAGES;
    extern __shared__ __align__(1024) unsigned char dsm[];
    float *estage = reinterpret_cast<float *>(dsm + STAGES * S::STAGE);
    __shared__ __align__(8) uint64_t full[STAGES], empty[STAGES], tfull[2], tempty[2];
    __shared__ uint32_t tmem_slot;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tiles_m = (M + TC_M - 1) / TC_M, tiles_n = (N + NT - 1) / NT;
    const long long tiles = (long long)tiles_m * tiles_n * batch;
    const int kblocks = (K + TP_KB - 1) / TP_KB;
    // FP32 row-major C whose rows start on 16-byte boundaries (BF16 outputs keep
    // the element-wise stores: their packing would not fit the register limit)
    const bool vec_rm = std::is_same<OUT, float>::value && c_cs == 1 && c_rs != 1 && c_rs % 4 == 0 &&
                        c_bs % 4 == 0 &&
                        (reinterpret_cast<uintptr_t>(C) % (4 * sizeof(OUT))) == 0 &&
                        (!EPI || !ep.vb || reinterpret_cast<uintptr_t>(ep.vb) % 8 == 0);

    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "r"((uint32_t)(2 * NT))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init_g(&full[s], 1);
            mbar_init_g(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init_g(&tfull[b], 1);
            mbar_init_g(&tempty[b], 8 * 32);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            long long it = 0;
            bool ok = true;
            for (long long t = blockIdx.x; t < tiles && ok; t += gridDim.x) {
                const int z = (int)(t / ((long long)tiles_m * tiles_n));
                const int rem = (int)(t - (long long)z * tiles_m * tiles_n);
                const int nt = rem / tiles_m, mt = rem - nt * tiles_m;
                for (int kb = 0; kb < kblocks; ++kb, ++it) {
                    const int s = (int)(it % STAGES);
                    const uint32_t ph = (uint32_t)(it / STAGES) & 1u;
                    if (!mbar_wait_g(&empty[s], ph ^ 1u, TC_WAIT)) {
                        atomicCAS(&g_gemm_status, 0, 2);
                        ok = false;
                        break;
                    }
                    mbar_expect_tx_g(&full[s], (uint32_t)S::STAGE);
                    unsigned char *sa = dsm + (size_t)s * S::STAGE, *sb = sa + S::A_BYTES;
                    if constexpr (AMN) {
                        tma_load_box(sa, &tmA, a3d != 0, mt * TC_M, kb * TP_KB, z, &full[s]);
                        tma_load_box(sa + S::A_BYTES / 2, &tmA, a3d != 0, mt * TC_M + 64, kb * TP_KB, z, &full[s]);
                    } else {
                        tma_load_box(sa, &tmA, a3d != 0, kb * TP_KB, mt * TC_M, z, &full[s]);
                    }
                    tma_load_box(sb, &tmB, b3d != 0, kb * TP_KB, nt * NT, z, &full[s]);
                }
            }
            // the copies of the last stages land before the CTA can exit
            for (long long j = it > STAGES ? it - STAGES : 0; j < it; ++j)
                mbar_wait_g(&full[j % STAGES], (uint32_t)(j / STAGES) & 1u, TC_WAIT);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            constexpr uint32_t idesc = umma_idesc_bf16(TC_M, NT) | (AMN ? (1u << 15) : 0u);  // bit 15: A MN-major
            long long it = 0;
            int tc = 0;
            bool ok = true;
            uint64_t *last = nullptr;  // the barrier of the last commit, and its phase
            uint32_t last_ph = 0;
            for (long long t = blockIdx.x; t < tiles && ok; t += gridDim.x, ++tc) {
                const int buf = tc & 1;
                const uint32_t aph = (uint32_t)(tc >> 1) & 1u;
                if (!mbar_wait_g(&tempty[buf], aph ^ 1u, TC_WAIT)) {
                    atomicCAS(&g_gemm_status, 0, 3);
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t d = tmem + (uint32_t)(buf * NT);
                for (int kb = 0; kb < kblocks; ++kb, ++it) {
                    const int s = (int)(it % STAGES);
                    const uint32_t ph = (uint32_t)(it / STAGES) & 1u;
                    if (!mbar_wait_g(&full[s], ph, TC_WAIT)) {
                        atomicCAS(&g_gemm_status, 0, 4);
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t sa = smem_u32(dsm + (size_t)s * S::STAGE), sb = sa + S::A_BYTES;
#pragma unroll
                    for (int kk = 0; kk < TP_KB / 16; ++kk) {
                        // K = 16 = 32 bytes of each 128-byte swizzled row; 8-row atoms 1024 bytes apart
                        const uint64_t da = AMN ? umma_desc(sa + kk * 2048, S::A_BYTES / 2, 1024, 2)
                                                : umma_desc(sa + kk * 32, 16, 1024, 2);
                        const uint64_t db = umma_desc(sb + kk * 32, 16, 1024, 2);
                        const uint32_t acc = (kb > 0 || kk > 0) ? 1u : 0u;
                        asm volatile(
                            "{\n\t.reg .pred p;\n\t"
                            "setp.ne.u32 p, %4, 0;\n\t"
                            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
                            "l"(da), "l"(db), "r"(idesc), "r"(acc)
                            : "memory");
                    }
                    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                     smem_u32(&empty[s]))
                                 : "memory");
                    last = &empty[s];
                    last_ph = ph;
                }
                if (!ok) break;
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 smem_u32(&tfull[buf]))
                             : "memory");
                last = &tfull[buf];  // completes phase tc >> 1 of tfull[buf]
                last_ph = aph;
            }
            // MMAs still in flight must finish before the tensor memory is freed
            if (last) mbar_wait_g(last, last_ph, TC_WAIT);
        }
    } else {
        const int ew = warp - 2, q = warp & 3, half = ew >> 2;
        float *ostage = estage + ew * (32 * 17);
        int tc = 0;
        for (long long t = blockIdx.x; t < tiles; t += gridDim.x, ++tc) {
            const int buf = tc & 1;
            const uint32_t ph = (uint32_t)(tc >> 1) & 1u;
            const bool w = mbar_wait_g(&tfull[buf], ph, TC_WAIT);
            if (!w) atomicCAS(&g_gemm_status, 0, 5);
            if (__any_sync(0xffffffffu, !w)) break;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int z = (int)(t / ((long long)tiles_m * tiles_n));
            const int rem = (int)(t - (long long)z * tiles_m * tiles_n);
            const int nt = rem / tiles_m, mt = rem - nt * tiles_m;
            const int m0 = mt * TC_M + q * 32, n0 = nt * NT;
            OUT *Cz = C + (long long)z * c_bs;
#pragma unroll 1
            for (int c0 = half * (NT / 2); c0 < (half + 1) * (NT / 2); c0 += 16) {
                uint32_t v[16];
                tc_ld16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(buf * NT + c0), v);
                if (std::is_same<OUT, float>::value && vec_rm && n0 + c0 + 16 <= N) {
                    // row-major C with aligned rows: stage the warp's 32 x 16
                    // block; a lane then owns four consecutive columns of
                    // rows 8i + lane/4 (16-byte loads and stores of C)
#pragma unroll
                    for (int j = 0; j < 16; ++j) ostage[lane * 17 + j] = __uint_as_float(v[j]);
                    __syncwarp();
                    const int quad = lane & 3, sub = lane >> 2, col = n0 + c0 + 4 * quad;
                    // EPI: the block's 32 rows meet at most one bias boundary
                    // when rows >= 32 (one division per block)
                    const long long b_lo = EPI && ep.rows >= 32 ? m0 / ep.rows : 0;
                    const long long edge = (b_lo + 1) * ep.rows;
                    // one row at a time: the kernel runs at its register
                    // limit (two CTAs of 320 threads per SM)
#pragma unroll 1
                    for (int i = 0; i < 4; ++i) {
                        const int r = 8 * i + sub, row = m0 + r;
                        if (row < M) {
                            OUT *p = Cz + (long long)row * c_rs + col;
                            float val[4] = {0.f, 0.f, 0.f, 0.f};
                            if (beta != 0.f) load4_out(p, val);
#pragma unroll
                            for (int e = 0; e < 4; ++e) val[e] = alpha * ostage[r * 17 + 4 * quad + e] + beta * val[e];
                            if (EPI && ep.bias) {
                                const float b = ep.bias[ep.rows >= 32 ? b_lo + (row >= edge) : row / ep.rows];
#pragma unroll
                                for (int e = 0; e < 4; ++e) val[e] = val[e] + b;
                            }
                            store4_out(p, val);
                            if (EPI && ep.vb) {
#pragma unroll
                                for (int e = 0; e < 4; ++e) val[e] = ep.act ? gelu_f(val[e]) : val[e];
                                *reinterpret_cast<uint2 *>(ep.vb + (long long)row * c_rs + col) = pack4_bf16(val);
                            }
                        }
                    }
                    __syncwarp();
                } else if (c_cs == 1 && c_rs != 1) {
                    // row-major C: stage the warp's 32 x 16 block and write two
                    // rows per instruction, 16 consecutive columns each
#pragma unroll
                    for (int j = 0; j < 16; ++j) ostage[lane * 17 + j] = __uint_as_float(v[j]);
                    __syncwarp();
                    const int j = lane & 15, col = n0 + c0 + j;
                    float old[16];
#pragma unroll
                    for (int i = 0; i < 16; ++i) {
                        const int row = m0 + 2 * i + (lane >> 4);
                        old[i] = (beta != 0.f && row < M && col < N) ? load_out(Cz + (long long)row * c_rs + col) : 0.f;
                    }
                    if (EPI && (ep.bias || ep.vb)) {
                        // the block's 32 rows meet at most one bias boundary
                        // when rows >= 32: one division per block
                        const long long b_lo = ep.rows >= 32 ? m0 / ep.rows : 0;
                        const long long edge = (b_lo + 1) * ep.rows;
#pragma unroll
                        for (int i = 0; i < 16; ++i) {
                            const int r = 2 * i + (lane >> 4), row = m0 + r;
                            if (row < M && col < N) {
                                float val = alpha * ostage[r * 17 + j] + beta * old[i];
                                if (ep.bias) {
                                    const long long bi = ep.rows >= 32 ? b_lo + (row >= edge) : row / ep.rows;
                                    val = val + ep.bias[bi];
                                }
                                store_out(Cz + (long long)row * c_rs + col, val);
                                if (ep.vb)
                                    ep.vb[(long long)row * c_rs + col] = __float2bfloat16_rn(ep.act ? gelu_f(val) : val);
                            }
                        }
                    } else {
#pragma unroll
                        for (int i = 0; i < 16; ++i) {
                            const int r = 2 * i + (lane >> 4), row = m0 + r;
                            if (row < M && col < N)
                                store_out(Cz + (long long)row * c_rs + col, alpha * ostage[r * 17 + j] + beta * old[i]);
                        }
                    }
                    __syncwarp();
                } else {
                    const int row = m0 + lane;
                    if (row < M) {
                        float old[16];
#pragma unroll
                        for (int j = 0; j < 16; ++j) {
                            const int col = n0 + c0 + j;
                            old[j] = (beta != 0.f && col < N) ? load_out(Cz + (long long)row * c_rs + (long long)col * c_cs)
                                                              : 0.f;
                        }
#pragma unroll
                        for (int j = 0; j < 16; ++j) {
                            const int col = n0 + c0 + j;
                            if (col < N)
                                store_out(Cz + (long long)row * c_rs + (long long)col * c_cs,
                                          alpha * __uint_as_float(v[j]) + beta * old[j]);
                        }
                    }
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            mbar_arrive_g(&tempty[buf]);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)(2 * NT))
                     : "memory");
}

// cuTensorMapEncodeTiled from the driver, looked up once through the runtime
// (the library links only the CUDA runtime)
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiledFn encode_tiled() {
    static std::atomic<EncodeTiledFn> fn{nullptr};
    static std::atomic<bool> tried{false};
    EncodeTiledFn f = fn.load(std::memory_order_acquire);
    if (f || tried.load(std::memory_order_acquire)) return f;
    std::lock_guard<std::mutex> lock(setup_mutex());
    if (!tried.load(std::memory_order_relaxed)) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn.store(reinterpret_cast<EncodeTiledFn>(p), std::memory_order_release);
        tried.store(true, std::memory_order_release);
    }
    return fn.load(std::memory_order_acquire);
}

// Tensor map of a K-major BF16 operand: rows x k, element (r, k) at
// X[r * rs + k], problem z at X + z * bs (3-D map when batch > 1 and bs != 0,
// else 2-D); box: 64 k (128 bytes, 128-byte swizzle) x box_rows rows.  False
// if TMA cannot address it.
static bool kmajor_map(CUtensorMap *map, const __nv_bfloat16 *X, long long rows, long long k, long long rs, int batch,
                       long long bs, int box_rows, int *three_d) {
    EncodeTiledFn enc = encode_tiled();
    if (!enc || !aligned(X, 16) || rs % 8 || rs <= 0 || bs % 8 || bs < 0 || k <= 0 || rows <= 0) return false;
    const bool use3 = batch > 1 && bs != 0;
    cuuint64_t dims[3] = {(cuuint64_t)k, (cuuint64_t)rows, (cuuint64_t)batch};
    cuuint64_t strides[2] = {(cuuint64_t)rs * 2, (cuuint64_t)bs * 2};
    cuuint32_t box[3] = {(cuuint32_t)TP_KB, (cuuint32_t)box_rows, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    const CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, use3 ? 3 : 2, const_cast<__nv_bfloat16 *>(X), dims,
                           strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    *three_d = use3 ? 1 : 0;
    return r == CUDA_SUCCESS;
}

// Tensor map of an M-major BF16 operand: element (m, k) at X[k * ks + m],
// problem z at X + z * bs; box: 64 m (128 bytes, 128-byte swizzle) x 64 k.
static bool mmajor_map(CUtensorMap *map, const __nv_bfloat16 *X, long long m, long long k, long long ks, int batch,
                       long long bs, int *three_d) {
    EncodeTiledFn enc = encode_tiled();
    if (!enc || !aligned(X, 16) || ks % 8 || ks <= 0 || bs % 8 || bs < 0 || k <= 0 || m <= 0) return false;
    const bool use3 = batch > 1 && bs != 0;
    cuuint64_t dims[3] = {(cuuint64_t)m, (cuuint64_t)k, (cuuint64_t)batch};
    cuuint64_t strides[2] = {(cuuint64_t)ks * 2, (cuuint64_t)bs * 2};
    cuuint32_t box[3] = {64, (cuuint32_t)TP_KB, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    const CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, use3 ? 3 : 2, const_cast<__nv_bfloat16 *>(X), dims,
                           strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    *three_d = use3 ? 1 : 0;
    return r == CUDA_SUCCESS;
}

// Launches the TMA pipeline if B is K-major, A K-major or M-major, and TMA
// can address them; returns 1 (nothing launched) when it cannot, so the
// caller falls back.
template <int NT, typename OUT>
static int launch_gemm_tma_nt(int m, int n, int k, const __nv_bfloat16 *a, long long a_rs, long long a_cs,
                              long long a_bs, const __nv_bfloat16 *b, long long b_cs, long long b_bs, OUT *C,
                              long long c_rs, long long c_cs, long long c_bs, int batch, float alpha, float beta,
                              const Epi &ep, cudaStream_t s) {
    using S = TmaShape<NT>;
    CUtensorMap ma, mb;
    int a3 = 0, b3 = 0;
    const bool amn = a_cs != 1;  // the caller passes a_cs == 1 (K-major) or a_rs == 1 (M-major)
    if (!(amn ? mmajor_map(&ma, a, m, k, a_cs, batch, a_bs, &a3) : kmajor_map(&ma, a, m, k, a_rs, batch, a_bs, TC_M, &a3)) ||
        !kmajor_map(&mb, b, n, k, b_cs, batch, b_bs, NT, &b3))
        return 1;
    const bool epi = ep.bias || ep.vb;
    if (epi && amn) return 1;  // the layer epilogue is built for a K-major A only
    // variants: K-major A, M-major A, K-major A with the layer epilogue
    static std::atomic<bool> attr[MAX_DEVICES][3];
    const int dev = current_device();
    const int variant = epi ? 2 : (amn ? 1 : 0);
    auto kernel_of = [](int v) {
        if constexpr (std::is_same<OUT, float>::value)
            if (v == 2) return k_gemm_tma<NT, OUT, false, true>;
        return v == 1 ? k_gemm_tma<NT, OUT, true, false> : k_gemm_tma<NT, OUT, false, false>;
    };
    if (epi && !std::is_same<OUT, float>::value) return 1;
    const auto kernel = kernel_of(variant);
    if (!attr[dev][variant].load(std::memory_order_acquire)) {
        std::lock_guard<std::mutex> lock(setup_mutex());
        const cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, S::SMEM);
        if (e != cudaSuccess) {
            set_error("k_gemm_tma: cannot reserve %d bytes of shared memory: %s", S::SMEM, cudaGetErrorString(e));
            return LBGB_ECUDA;
        }
        attr[dev][variant].store(true, std::memory_order_release);
    }
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long tiles = (long long)((m + TC_M - 1) / TC_M) * ((n + NT - 1) / NT) * batch;
    const long long slots = 2ll * (sms > 0 ? sms : 1);
    const int grid = (int)(tiles < slots ? tiles : slots);
    kernel<<<grid, TP_THREADS, S::SMEM, s>>>(ma, mb, a3, b3, m, n, k, batch, C, c_rs, c_cs, c_bs, alpha, beta, ep);
    return check_launch("k_gemm_tma");
}

template <typename OUT>
static int launch_gemm_tma(int m, int n, int k, const __nv_bfloat16 *a, long long a_rs, long long a_cs, long long a_bs,
                           const __nv_bfloat16 *b, long long b_rs, long long b_cs, long long b_bs, OUT *C,
                           long long c_rs, long long c_cs, long long c_bs, int batch, float alpha, float beta,
                           bool forced, cudaStream_t s, const Epi &ep = Epi()) {
    if ((a_cs != 1 && a_rs != 1) || b_rs != 1 || k <= 0) return 1;
    // automatic choice: M-major A with more than 64 output columns stays on
    // the staged kernel -- there the output (the 128-channel projection:
    // 512 MB per pass) is what takes the time, and 8192 staged CTAs drain it
    // faster than the persistent kernel's two CTAs per SM (119 against 192 us)
    if (!forced && a_cs != 1 && n > 64) return 1;
    if (n <= 32)
        return launch_gemm_tma_nt<32>(m, n, k, a, a_rs, a_cs, a_bs, b, b_cs, b_bs, C, c_rs, c_cs, c_bs, batch, alpha,
                                      beta, ep, s);
    if (n <= 64)
        return launch_gemm_tma_nt<64>(m, n, k, a, a_rs, a_cs, a_bs, b, b_cs, b_bs, C, c_rs, c_cs, c_bs, batch, alpha,
                                      beta, ep, s);
    return launch_gemm_tma_nt<128>(m, n, k, a, a_rs, a_cs, a_bs, b, b_cs, b_bs, C, c_rs, c_cs, c_bs, batch, alpha,
                                   beta, ep, s);
}

template <typename OUT>
static int launch_gemm(int m, int n, int k, const __nv_bfloat16 *a, long long a_rs, long long a_cs, long long a_bs,
                       const __nv_bfloat16 *b, long long b_rs, long long b_cs, long long b_bs, OUT *C, long long c_rs,
                       long long c_cs, long long c_bs, int batch, float alpha, float beta, int engine,
                       cudaStream_t s) {
    if (engine == 0 || engine == 3) {
        // both operands K-major: the TMA pipeline (engine 3 insists on it)
        const int rc = k > 0 ? launch_gemm_tma(m, n, k, a, a_rs, a_cs, a_bs, b, b_rs, b_cs, b_bs, C, c_rs, c_cs, c_bs,
                                               batch, alpha, beta, engine == 3, s)
                             : 1;
        if (rc <= 0) return rc;
        if (engine == 3) {
            set_error("lbgb_gemm_bf16: engine 3 needs a K-major B, a K- or M-major A and 16-byte aligned rows");
            return LBGB_EINVAL;
        }
    }
    if (engine == 1 || k == 0) {  // K = 0: C = beta C, no tensor-core work
        dim3 grid((m + 63) / 64, (n + 63) / 64, batch);
        k_gemm_simt<OUT><<<grid, 256, 0, s>>>(m, n, k, a, a_rs, a_cs, a_bs, b, b_rs, b_cs, b_bs, C, c_rs, c_cs, c_bs,
                                              alpha, beta);
        return check_launch("k_gemm_simt");
    }
    // tensor cores: tile N 32/64/128 by problem width; K blocks of 32 when K
    // is that small (most of the surrogate's products), else 64.  One operand
    // stage: double-buffering the K blocks (ST = 2, the loads of block kb
    // under the MMAs of kb-1) measured slower on the surrogate's products
    // (training step 6.81 ms for K > 64, 6.75 ms for K > 192, 6.54 ms never)
    // -- the larger shared-memory footprint costs more resident CTAs than the
    // overlap gains.
    dim3 grid((m + TC_M - 1) / TC_M, 1, batch);
#define LBGB_TC(NTV, KBV, STV)                                                                                   \
    do {                                                                                                       \
        grid.y = (n + NTV - 1) / NTV;                                                                          \
        const int dyn = tc_dyn_smem<NTV, OUT, KBV, STV>();                                                     \
        k_gemm_tc<NTV, OUT, KBV, STV><<<grid, 128, dyn, s>>>(m, n, k, a, a_rs, a_cs, a_bs, b, b_rs, b_cs, b_bs, C, \
                                                             c_rs, c_cs, c_bs, alpha, beta);                  \
    } while (0)
#define LBGB_TC_K(NTV)                                                                                         \
    do {                                                                                                       \
        if (k <= 32) LBGB_TC(NTV, 32, 1);                                                                      \
        else LBGB_TC(NTV, 64, 1);                                                                              \
    } while (0)
    if (n <= 32) LBGB_TC_K(32);
    else if (n <= 64) LBGB_TC_K(64);
    else LBGB_TC_K(128);
#undef LBGB_TC_K
#undef LBGB_TC
    return check_launch("k_gemm_tc");
}

}  // namespace lbgb

using namespace lbgb;

extern "C" int lbgb_gemm_bf16(int m, int n, int k, const void *A, long long a_rs, long long a_cs, long long a_bs,
                              const void *B, long long b_rs, long long b_cs, long long b_bs, void *C, long long c_rs,
                              long long c_cs, long long c_bs, int batch, float alpha, float beta, int c_bf16,
                              int engine, void *stream) {
    if (m < 0 || n < 0 || k < 0 || batch < 1 || batch > 65535) {
        set_error("lbgb_gemm_bf16: bad sizes m=%d n=%d k=%d batch=%d", m, n, k, batch);
        return LBGB_EINVAL;
    }
    if (m == 0 || n == 0) return LBGB_OK;
    if (!C || (k > 0 && (!A || !B))) {
        set_error("lbgb_gemm_bf16: null operand");
        return LBGB_EINVAL;
    }
    if (engine < 0 || engine > 3) {
        set_error("lbgb_gemm_bf16: unknown engine %d", engine);
        return LBGB_EINVAL;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const auto *a = static_cast<const __nv_bfloat16 *>(A);
    const auto *b = static_cast<const __nv_bfloat16 *>(B);
    if (c_bf16)
        return launch_gemm(m, n, k, a, a_rs, a_cs, a_bs, b, b_rs, b_cs, b_bs, static_cast<__nv_bfloat16 *>(C), c_rs,
                           c_cs, c_bs, batch, alpha, beta, engine, s);
    return launch_gemm(m, n, k, a, a_rs, a_cs, a_bs, b, b_rs, b_cs, b_bs, static_cast<float *>(C), c_rs, c_cs, c_bs,
                       batch, alpha, beta, engine, s);
}

extern "C" int lbgb_gemm_bf16_bias_act(int m, int n, int k, const void *A, long long a_rs, long long a_cs,
                                       const void *B, long long b_cs, void *C, long long c_rs, float alpha, float beta,
                                       const float *bias, long long rows_per_bias, int act, void *c_bf16_copy,
                                       void *stream) {
    if (m <= 0 || n <= 0 || k <= 0 || rows_per_bias <= 0 || !A || !B || !C) {
        set_error("lbgb_gemm_bf16_bias_act: bad sizes or operands (m=%d n=%d k=%d rows_per_bias=%lld)", m, n, k,
                  rows_per_bias);
        return LBGB_EINVAL;
    }
    if (a_cs != 1 || c_rs < n || c_rs <= 1 || !aligned(C, 16) || (c_bf16_copy && !aligned(c_bf16_copy, 16))) {
        set_error("lbgb_gemm_bf16_bias_act: needs a K-major A and a row-major C (16-byte aligned)");
        return LBGB_EUNSUPPORTED;
    }
    Epi ep;
    ep.bias = bias;
    ep.rows = rows_per_bias;
    ep.act = act;
    ep.vb = static_cast<__nv_bfloat16 *>(c_bf16_copy);
    const int rc = launch_gemm_tma(m, n, k, static_cast<const __nv_bfloat16 *>(A), a_rs, a_cs, 0,
                                   static_cast<const __nv_bfloat16 *>(B), 1, b_cs, 0, static_cast<float *>(C), c_rs, 1,
                                   0, 1, alpha, beta, true, (cudaStream_t)stream, ep);
    if (rc > 0) {
        set_error("lbgb_gemm_bf16_bias_act: the TMA pipeline cannot address these operands");
        return LBGB_EUNSUPPORTED;
    }
    return rc;
}

extern "C" int lbgb_gemm_status(int reset) {
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        set_error("lbgb_gemm_status: %s", cudaGetErrorString(e));
        return LBGB_ECUDA;
    }
    int v = 0;
    e = cudaMemcpyFromSymbol(&v, g_gemm_status, sizeof(int));
    if (e == cudaSuccess && reset) {
        const int zero = 0;
        e = cudaMemcpyToSymbol(g_gemm_status, &zero, sizeof(int));
    }
    if (e != cudaSuccess) {
        set_error("lbgb_gemm_status: %s", cudaGetErrorString(e));
        return LBGB_ECUDA;
    }
    if (v) {
        set_error("a bounded wait in the tensor-core GEMM gave up");
        return LBGB_ETIMEOUT;
    }
    return LBGB_OK;
}
