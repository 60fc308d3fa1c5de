// Shared device code of liblbgb: D2Q9 constants, population storage codecs,
// vector memory access and the BGK collision of one node.
#pragma once

#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>
#include <stdint.h>
#include <string.h>

#include <atomic>
#include <mutex>

#include "lbgb.h"

namespace lbgb {

// ---------------------------------------------------------------- lattice
// Channel order 0, E, N, W, S, NE, NW, SW, SE (PyLB/Streaming.py:28-29).
enum { C0 = 0, CE = 1, CN = 2, CW = 3, CS = 4, CNE = 5, CNW = 6, CSW = 7, CSE = 8 };

__host__ __device__ constexpr int cx(int i) {
    return (i == CE || i == CNE || i == CSE) ? 1 : (i == CW || i == CNW || i == CSW) ? -1 : 0;
}
__host__ __device__ constexpr int cy(int i) {
    return (i == CN || i == CNE || i == CNW) ? 1 : (i == CS || i == CSW || i == CSE) ? -1 : 0;
}
__host__ __device__ constexpr int opp(int i) {
    return i == 0 ? 0 : (i <= 4 ? (i + 1) % 4 + 1 : (i - 3) % 4 + 5);
}
// Lattice weights 4/9, 1/9, 1/36 (cavity_opt1.py:92-96).  Opposite channels
// share a weight, which the bounce-back decode below relies on.
template <class R>
__host__ __device__ constexpr R wgt(int i) {
    return i == 0 ? R(4.0 / 9.0) : (i <= 4 ? R(1.0 / 9.0) : R(1.0 / 36.0));
}

// ---------------------------------------------------------------- storage
// raw = element type in HBM, real = arithmetic type.  The deviation codecs
// store h_i = f_i - w_i as 16-bit bits (IEEE half or bfloat16).
template <int DT> struct Codec;

// DEV: the kernels' values are deviations h_i = f_i - w_i (LBGB_F32DEV and the
// two 16-bit codecs) rather than populations; decd/encd convert to and from
// the population in FP64.
template <> struct Codec<LBGB_F32> {
    using raw = float;
    using real = float;
    static constexpr bool DEV = false;
    static __device__ __forceinline__ real dec(raw x, int) { return x; }
    static __device__ __forceinline__ raw enc(real x, int) { return x; }
    static __device__ __forceinline__ double decd(raw x, int) { return x; }
    static __device__ __forceinline__ raw encd(double f, int) { return (raw)f; }
};
template <> struct Codec<LBGB_F64> {
    using raw = double;
    using real = double;
    static constexpr bool DEV = false;
    static __device__ __forceinline__ real dec(raw x, int) { return x; }
    static __device__ __forceinline__ raw enc(real x, int) { return x; }
    static __device__ __forceinline__ double decd(raw x, int) { return x; }
    static __device__ __forceinline__ raw encd(double f, int) { return f; }
};
template <> struct Codec<LBGB_F32DEV> {
    using raw = float;
    using real = float;
    static constexpr bool DEV = true;
    static __device__ __forceinline__ real dec(raw x, int) { return x; }
    static __device__ __forceinline__ raw enc(real x, int) { return x; }
    static __device__ __forceinline__ double decd(raw x, int i) { return (double)x + wgt<double>(i); }
    static __device__ __forceinline__ raw encd(double f, int i) { return (raw)(f - wgt<double>(i)); }
};
// Half deviations are stored scaled by 2^14: deviations down to ~4e-9 stay
// in half's normal range (full 11-bit precision instead of the coarse
// subnormal grid below 6e-5), and |f - w| < 4 still fits.  Scaling by a power
// of two is exact in both directions.
constexpr float F16_SCALE = 16384.0f;
constexpr float F16_UNSCALE = 1.0f / 16384.0f;

// Mixed-precision FMA with 16-bit multiplicands (PTX fma.rn.f32.f16 and
// fma.rn.f32.bf16, sm_100 and later): a b + c for 16-bit a, b and an FP32
// addend, rounded once to FP32.  The result is the fmaf of the exactly
// converted operands, in one instruction instead of a conversion and an FMA.
constexpr unsigned short F16_UNSCALE_BITS = 0x0400;    // half 2^-14
constexpr unsigned short F16_MINUS_ONE_BITS = 0xbc00;  // half -1
constexpr unsigned short F16_ONE_BITS = 0x3c00;        // half 1
template <bool BF>
__device__ __forceinline__ float fma16(unsigned short a, unsigned short b, float c) {
    float d;
    if constexpr (BF)
        asm("fma.rn.f32.bf16 %0, %1, %2, %3;" : "=f"(d) : "h"(a), "h"(b), "f"(c));
    else
        asm("fma.rn.f32.f16 %0, %1, %2, %3;" : "=f"(d) : "h"(a), "h"(b), "f"(c));
    return d;
}
// the two 16-bit values of a 32-bit word (low half first), each times b plus
// its own addend
template <bool BF>
__device__ __forceinline__ void fma16x2(uint32_t a2, unsigned short b, float c_lo, float c_hi, float &lo,
                                        float &hi) {
    if constexpr (BF)
        asm("{\n\t.reg .b16 l, h;\n\tmov.b32 {l, h}, %2;\n\t"
            "fma.rn.f32.bf16 %0, l, %3, %4;\n\tfma.rn.f32.bf16 %1, h, %3, %5;\n\t}"
            : "=f"(lo), "=f"(hi) : "r"(a2), "h"(b), "f"(c_lo), "f"(c_hi));
    else
        asm("{\n\t.reg .b16 l, h;\n\tmov.b32 {l, h}, %2;\n\t"
            "fma.rn.f32.f16 %0, l, %3, %4;\n\tfma.rn.f32.f16 %1, h, %3, %5;\n\t}"
            : "=f"(lo), "=f"(hi) : "r"(a2), "h"(b), "f"(c_lo), "f"(c_hi));
}

// The 16-bit codecs are DEV codecs too: the kernels work on h = f - w_i, the
// collision in deviation form (collide_dev), so that no population is ever
// rebuilt from its weight and every rounding acts on a small number.
template <> struct Codec<LBGB_F16DEV> {
    using raw = unsigned short;
    using real = float;
    static constexpr bool DEV = true;
    static __device__ __forceinline__ real dec_h(raw x) { return fma16<false>(x, F16_UNSCALE_BITS, 0.f); }
    static __device__ __forceinline__ raw enc_h(real h) { return __half_as_ushort(__float2half_rn(h * F16_SCALE)); }
    static __device__ __forceinline__ real dec(raw x, int) { return dec_h(x); }
    static __device__ __forceinline__ raw enc(real h, int) { return enc_h(h); }
    static __device__ __forceinline__ double decd(raw x, int i) { return (double)dec_h(x) + wgt<double>(i); }
    static __device__ __forceinline__ raw encd(double f, int i) { return enc_h((real)(f - wgt<double>(i))); }
};
template <> struct Codec<LBGB_BF16DEV> {
    using raw = unsigned short;
    using real = float;
    static constexpr bool DEV = true;
    static __device__ __forceinline__ real dec_h(raw x) { return __uint_as_float((uint32_t)x << 16); }
    static __device__ __forceinline__ raw enc_h(real h) { return __bfloat16_as_ushort(__float2bfloat16_rn(h)); }
    static __device__ __forceinline__ real dec(raw x, int) { return dec_h(x); }
    static __device__ __forceinline__ raw enc(real h, int) { return enc_h(h); }
    static __device__ __forceinline__ double decd(raw x, int i) { return (double)dec_h(x) + wgt<double>(i); }
    static __device__ __forceinline__ raw encd(double f, int i) { return enc_h((real)(f - wgt<double>(i))); }
};

// Density of a node from its nine kernel values (populations, or deviations
// for DEV codecs: 1 + sum h, the small numbers summed first).
template <int DT>
__device__ __forceinline__ typename Codec<DT>::real node_density(const typename Codec<DT>::real (&v)[9]) {
    typename Codec<DT>::real r = v[0];
#pragma unroll
    for (int i = 1; i < 9; ++i) r += v[i];
    if constexpr (Codec<DT>::DEV) r += typename Codec<DT>::real(1);
    return r;
}

// ---------------------------------------------------------------- memory
// A vector of V raw elements moved as one 2/4/8/16-byte access.
template <int BYTES> struct VecBits;
template <> struct VecBits<16> { using t = uint4; };
template <> struct VecBits<8> { using t = uint2; };
template <> struct VecBits<4> { using t = unsigned int; };
template <> struct VecBits<2> { using t = unsigned short; };

// Read-only, non-coherent load (src is never written by the same launch).
template <class RAW, int V>
__device__ __forceinline__ void ldv(const RAW *p, RAW (&o)[V]) {
    using T = typename VecBits<V * sizeof(RAW)>::t;
    T x = __ldg(reinterpret_cast<const T *>(p));
    memcpy(o, &x, sizeof(T));
}

template <class RAW>
__device__ __forceinline__ RAW ld1(const RAW *p) {
    RAW o[1];
    ldv<RAW, 1>(p, o);
    return o[0];
}

// Streaming store: the written populations are not re-read by this launch.
__device__ __forceinline__ void st_cs(uint4 *p, uint4 v) {
    asm volatile("st.global.cs.v4.u32 [%0], {%1, %2, %3, %4};" ::"l"(p), "r"(v.x), "r"(v.y),
                 "r"(v.z), "r"(v.w) : "memory");
}
__device__ __forceinline__ void st_cs(uint2 *p, uint2 v) {
    asm volatile("st.global.cs.v2.u32 [%0], {%1, %2};" ::"l"(p), "r"(v.x), "r"(v.y) : "memory");
}
__device__ __forceinline__ void st_cs(unsigned int *p, unsigned int v) {
    asm volatile("st.global.cs.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void st_cs(unsigned short *p, unsigned short v) {
    asm volatile("st.global.cs.u16 [%0], %1;" ::"l"(p), "h"(v) : "memory");
}

template <class RAW, int V>
__device__ __forceinline__ void stv(RAW *p, const RAW (&v)[V]) {
    using T = typename VecBits<V * sizeof(RAW)>::t;
    T x;
    memcpy(&x, v, sizeof(T));
    st_cs(reinterpret_cast<T *>(p), x);
}

// ---------------------------------------------------------------- packets
// A packet is the N consecutive cells of one channel that one thread moves as
// one 8- or 16-byte vector.  The 16-bit routines convert two values per
// instruction where the hardware allows (float2 -> half2 / bfloat162); the
// decode folds each 16-bit value into its FMA (fma16x2).
template <int DT, int N>
struct Packet {
    using raw = typename Codec<DT>::raw;
    using real = typename Codec<DT>::real;
    static constexpr int BYTES = N * (int)sizeof(raw);
    static constexpr int WORDS = BYTES / 4;
    using vec = typename VecBits<BYTES>::t;

    // the kernel values of a packet: f (FP32, FP64) or h = f - w (the DEV
    // codecs); w is unused (the weights never enter a decode)
    static __device__ __forceinline__ void dec(const vec &x, real, real (&o)[N]) {
        uint32_t wd[WORDS];
        memcpy(wd, &x, BYTES);
        if constexpr (DT == LBGB_F32 || DT == LBGB_F32DEV) {
#pragma unroll
            for (int q = 0; q < N; ++q) o[q] = __uint_as_float(wd[q]);
        } else if constexpr (DT == LBGB_F64) {
#pragma unroll
            for (int q = 0; q < N; ++q) o[q] = __hiloint2double((int)wd[2 * q + 1], (int)wd[2 * q]);
        } else {
#pragma unroll
            for (int q = 0; q < WORDS; ++q) {
                if constexpr (DT == LBGB_F16DEV) {
                    fma16x2<false>(wd[q], F16_UNSCALE_BITS, 0.f, 0.f, o[2 * q], o[2 * q + 1]);
                } else {
                    o[2 * q] = __uint_as_float(wd[q] << 16);
                    o[2 * q + 1] = __uint_as_float(wd[q] & 0xffff0000u);
                }
            }
        }
    }
    // the kernel value of one stored element (w unused, as in dec)
    static __device__ __forceinline__ real dec1(raw x, real) {
        if constexpr (DT == LBGB_F16DEV || DT == LBGB_BF16DEV)
            return Codec<DT>::dec_h(x);
        else
            return x;
    }
    // the stored 16-bit values of a packet as FP32 without unscaling (FP16:
    // the deviation times 2^14, exactly; bfloat16: the deviation)
    static __device__ __forceinline__ void dec_units(const vec &x, real (&o)[N]) {
        uint32_t wd[WORDS];
        memcpy(wd, &x, BYTES);
#pragma unroll
        for (int q = 0; q < WORDS; ++q) {
            if constexpr (DT == LBGB_F16DEV) {
                fma16x2<false>(wd[q], F16_ONE_BITS, 0.f, 0.f, o[2 * q], o[2 * q + 1]);
            } else {
                o[2 * q] = __uint_as_float(wd[q] << 16);
                o[2 * q + 1] = __uint_as_float(wd[q] & 0xffff0000u);
            }
        }
    }
    static __device__ __forceinline__ real dec1_units(raw x) {
        if constexpr (DT == LBGB_F16DEV)
            return __half2float(__ushort_as_half(x));
        else
            return Codec<DT>::dec_h(x);
    }
    // packs N FP16 values that are already scaled by 2^14, two per conversion
    static __device__ __forceinline__ vec enc_scaled(const real (&hs)[N]) {
        uint32_t wd[WORDS];
#pragma unroll
        for (int q = 0; q < WORDS; ++q) {
            const __half2 p = __floats2half2_rn(hs[2 * q], hs[2 * q + 1]);
            wd[q] = *reinterpret_cast<const uint32_t *>(&p);
        }
        vec x;
        memcpy(&x, wd, BYTES);
        return x;
    }
    // packs N deviations of a 16-bit codec, two per conversion
    static __device__ __forceinline__ vec enc_h(const real (&h)[N]) {
        uint32_t wd[WORDS];
#pragma unroll
        for (int q = 0; q < WORDS; ++q) {
            if constexpr (DT == LBGB_F16DEV) {
                const __half2 p = __floats2half2_rn(h[2 * q] * F16_SCALE, h[2 * q + 1] * F16_SCALE);
                wd[q] = *reinterpret_cast<const uint32_t *>(&p);
            } else {
                const __nv_bfloat162 p = __floats2bfloat162_rn(h[2 * q], h[2 * q + 1]);
                wd[q] = *reinterpret_cast<const uint32_t *>(&p);
            }
        }
        vec x;
        memcpy(&x, wd, BYTES);
        return x;
    }
};



// ---------------------------------------------------------------- stochastic rounding
// Rounding a slowly varying field to 16 bits repeats the same error at every
// step, so the errors add up linearly (mass and momentum drift).  Stochastic
// rounding -- round up with probability equal to the discarded fraction --
// makes every rounding unbiased, and the accumulated error a random walk.
// The random bits are a counter-based hash of (seed, step, cell, channel), so
// every kernel variant rounds every value identically.  Two neighbouring
// cells (2m, 2m+1) of a channel share one 32-bit word: one hash of the pair
// and the step key, then per channel a multiply by an odd multiplier of the
// channel's own and an xorshift (both bijections, so the word stays uniform;
// the high word of the product alone would not be: it is below the
// multiplier, and biased rounding follows).  The rounding itself is the hardware's stochastic
// conversion (cvt.rs.{f16x2,bf16x2}.f32, sm_100 and later), which rounds the
// even cell with bits 15:0 and the odd cell with bits 31:16 of the word.
__host__ __device__ constexpr uint32_t mix32(uint32_t x) {
    // integer finaliser with the constants of the public-domain "lowbias32"
    // from C. Wellons' hash-prospector
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}
__device__ __forceinline__ uint32_t sr_step_key(uint32_t seed, unsigned long long step) {
    return mix32(seed ^ mix32((uint32_t)step * 0x9e3779b9u + (uint32_t)(step >> 32)));
}
__device__ __forceinline__ uint32_t sr_pair_base(uint32_t key, uint32_t even_cell) { return mix32(even_cell ^ key); }
__host__ __device__ constexpr uint32_t sr_mult(int ch) { return mix32(0x9e3779b9u * (uint32_t)(ch + 1)) | 1u; }
__device__ __forceinline__ uint32_t sr_channel_bits(uint32_t base, int ch) {
    const uint32_t x = base * sr_mult(ch);
    return x ^ (x >> 16);
}
// two FP32 values -> one word of two 16-bit codes, stochastically rounded:
// lo to bits 15:0 (random bits r[15:0]), hi to bits 31:16 (r[31:16]).
// Half codes take the deviation already scaled by 2^14 (sr_dev).
template <int DT>
__device__ __forceinline__ uint32_t sr_pack2(float lo, float hi, uint32_t r) {
    uint32_t d;
    if constexpr (DT == LBGB_BF16DEV)
        asm("cvt.rs.bf16x2.f32 %0, %1, %2, %3;" : "=r"(d) : "f"(hi), "f"(lo), "r"(r));
    else
        asm("cvt.rs.f16x2.f32 %0, %1, %2, %3;" : "=r"(d) : "f"(hi), "f"(lo), "r"(r));
    return d;
}
// the value that sr_pack2 rounds for deviation h: h, or h 2^14 for half codes
template <int DT>
__device__ __forceinline__ float sr_dev(float h) {
    if constexpr (DT == LBGB_BF16DEV)
        return h;
    else
        return h * F16_SCALE;
}
// the same for the rest population's remaining mass deviation d
template <int DT>
__device__ __forceinline__ float sr_rest(float d) {
    if constexpr (DT == LBGB_BF16DEV)
        return d;
    else
        return d * F16_SCALE;
}
// d minus the deviation that a stored 16-bit code carries, one instruction
// per value (the code times -1, or -2^-14 for scaled half, plus d)
constexpr unsigned short F16_MINUS_UNSCALE_BITS = 0x8400;  // half -2^-14
constexpr unsigned short BF16_MINUS_ONE_BITS = 0xbf80;     // bfloat16 -1
template <int DT>
__device__ __forceinline__ float sub_stored(float d, unsigned short x) {
    if constexpr (DT == LBGB_BF16DEV)
        return fma16<true>(x, BF16_MINUS_ONE_BITS, d);
    else
        return fma16<false>(x, F16_MINUS_UNSCALE_BITS, d);
}
template <int DT>
__device__ __forceinline__ void sub_stored2(float &d_lo, float &d_hi, uint32_t w) {
    if constexpr (DT == LBGB_BF16DEV)
        fma16x2<true>(w, BF16_MINUS_ONE_BITS, d_lo, d_hi, d_lo, d_hi);
    else
        fma16x2<false>(w, F16_MINUS_UNSCALE_BITS, d_lo, d_hi, d_lo, d_hi);
}

// packs N deviations of a 16-bit codec with stochastic rounding; base[q] is
// sr_pair_base of the packet's cell pair q
template <int DT, int N>
__device__ __forceinline__ typename Packet<DT, N>::vec enc_h_sr(const float (&h)[N], const uint32_t (&base)[N / 2],
                                                              int ch) {
    using P = Packet<DT, N>;
    uint32_t wd[P::WORDS];
#pragma unroll
    for (int q = 0; q < P::WORDS; ++q) wd[q] = sr_pack2<DT>(h[2 * q], h[2 * q + 1], sr_channel_bits(base[q], ch));
    typename P::vec x;
    memcpy(&x, wd, P::BYTES);
    return x;
}

// ---------------------------------------------------------------- collision
// BGK relaxation of one node towards the D2Q9 equilibrium
//   f_i += omega (w_i rho (1 + 3 c.u + 9/2 (c.u)^2 - 3/2 u^2) - f_i),
// in the formulation of c/d2q9.h:59-81,121-131: rho = sum f, u = sum c f / rho,
// ux, uy scaled by 3, uu = (ux^2 + uy^2)/6, feq_i = w_i rho (1 + cu + cu^2/2 - uu).
__device__ __forceinline__ float recip(float x) { return __frcp_rn(x); }
__device__ __forceinline__ double recip(double x) { return __drcp_rn(x); }
// hardware reciprocal approximation (one MUFU op, ~1 ulp): for 16-bit storage,
// whose own rounding is 2^-11 or coarser
__device__ __forceinline__ float recip_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// BGK relaxation of one node with its density already summed.
template <class R>
__device__ __forceinline__ void bgk_relax(R (&f)[9], R omega, R rho, R &ux_out, R &uy_out) {
    const R inv = recip(rho);
    R ux = (f[1] - f[3] + f[5] - f[6] - f[7] + f[8]) * inv;
    R uy = (f[2] - f[4] + f[5] + f[6] - f[7] - f[8]) * inv;
    ux_out = ux;
    uy_out = uy;
    const R w0 = rho * R(4.0 / 9.0), w1 = rho * R(1.0 / 9.0), w5 = rho * R(1.0 / 36.0);
    ux *= R(3);
    uy *= R(3);
    const R uu = (ux * ux + uy * uy) * R(1.0 / 6.0);
    const R base = R(1) - uu;
    const R cu5 = ux + uy, cu6 = uy - ux;
    const R hx = R(0.5) * ux * ux, hy = R(0.5) * uy * uy;
    const R h5 = R(0.5) * cu5 * cu5, h6 = R(0.5) * cu6 * cu6;
    R feq[9];
    feq[0] = w0 * base;
    feq[1] = w1 * (base + ux + hx);
    feq[2] = w1 * (base + uy + hy);
    feq[3] = w1 * (base - ux + hx);
    feq[4] = w1 * (base - uy + hy);
    feq[5] = w5 * (base + cu5 + h5);
    feq[6] = w5 * (base + cu6 + h6);
    feq[7] = w5 * (base - cu5 + h5);
    feq[8] = w5 * (base - cu6 + h6);
#pragma unroll
    for (int i = 0; i < 9; ++i) f[i] += omega * (feq[i] - f[i]);
}

template <class R>
__device__ __forceinline__ void bgk_collide(R (&f)[9], R omega, R &rho_out, R &ux_out, R &uy_out) {
    R rho = f[0];
#pragma unroll
    for (int i = 1; i < 9; ++i) rho += f[i];
    rho_out = rho;
    bgk_relax(f, omega, rho, ux_out, uy_out);
}

template <class R>
__device__ __forceinline__ void bgk_collide(R (&f)[9], R omega) {
    R a, b, c;
    bgk_collide(f, omega, a, b, c);
}

// IEEE operations rounded one by one: the compiler may not contract them into
// FMAs or replace a division by a reciprocal multiply.
template <class R> struct Ieee;
template <> struct Ieee<float> {
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
    static __device__ __forceinline__ float fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
    static __device__ __forceinline__ float rcp(float b) { return __frcp_rn(b); }
    // operand ranges of the reciprocal division below (no intermediate
    // overflows or leaves the normal range)
    static constexpr float A_MIN = 0x1p-60f, A_MAX = 0x1p60f, B_MIN = 0x1p-30f, B_MAX = 0x1p30f;
};
template <> struct Ieee<double> {
    static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
    static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
    static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
    static __device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
    static __device__ __forceinline__ double fma(double a, double b, double c) { return __fma_rn(a, b, c); }
    static __device__ __forceinline__ double rcp(double b) { return __drcp_rn(b); }
    static constexpr double A_MIN = 0x1p-500, A_MAX = 0x1p500, B_MIN = 0x1p-250, B_MAX = 0x1p250;
};

// The correctly rounded quotient RN(a / b) from y = RN(1/b), by Markstein's
// correction (P. Markstein, "Computation of elementary functions on the IBM
// RISC System/6000 processor", IBM J. Res. Develop. 34, 1990; J.-M. Muller et
// al., Handbook of Floating-Point Arithmetic, ch. on division by FMA):
//   q0 = RN(a y), within 1.5 ulp of a/b;
//   r0 = a - b q0 (exact: one FMA), q1 = RN(q0 + r0 y), within one ulp;
//   r1 = a - b q1 (exact), q2 = RN(q1 + r1 y) = RN(a / b),
// the last step by Markstein's theorem (y within half an ulp of 1/b, q1
// within one ulp of a/b, no underflow or overflow).  Outside the operand
// range where that holds, and for b out of range, the IEEE division itself;
// a = +-0 gives a y, the correctly signed zero.  Same result as Ieee<R>::div
// for every input, at a few FMAs instead of a division per quotient.
template <class R>
__device__ __forceinline__ R div_by_rcp(R a, R b, R y) {
    using O = Ieee<R>;
    const R aa = a < R(0) ? -a : a, ab = b < R(0) ? -b : b;
    const bool b_ok = ab >= O::B_MIN && ab <= O::B_MAX;
    if (b_ok && aa >= O::A_MIN && aa <= O::A_MAX) {
        const R q0 = O::mul(a, y);
        const R q1 = O::fma(O::fma(-b, q0, a), y, q0);
        return O::fma(O::fma(-b, q1, a), y, q1);
    }
    if (b_ok && a == R(0)) return O::mul(a, y);
    return O::div(a, b);
}

// The BGK collision of the reference's native kernel, operation by operation
// (d2q9_colliden, c/d2q9.h:121-131, with d2q9_equilibrium1, c/d2q9.h:59-81):
//   rho = f_i.sum()  -- Eigen 3.4 reduces a fixed-size 9-vector by an
//                       unrolled halving split: ((f0+f1)+(f2+f3)) +
//                       ((f4+f5)+(f6+(f7+f8)))
//   ux = (f1-f3+f5-f6-f7+f8)/rho, uy = (f2-f4+f5+f6-f7-f8)/rho (left to right)
//   w0 = 4 rho/9, w1 = rho/9, w5 = rho/36; ux *= 3; uy *= 3
//   uu = (ux ux + uy uy)/6; feq_i = w_i (((1 + cu) + cu cu/2) - uu)
//   f_i += omega (feq_i - f_i)
// Every operation is rounded on its own (the x86-64 build of the reference
// has no FMA), so FP32 and FP64 results equal the native kernel's bit for bit.
// d2q9_equilibrium1 (c/d2q9.h:59-81) operation by operation.
// The divisions are the IEEE ones, computed faster with the same results:
// by a constant through its correctly rounded reciprocal (div_by_rcp), and
// x / 2 as x * 0.5 (both are the one rounding of the exact x/2).
template <class R>
__device__ __forceinline__ void equilibrium_native(R rho, R ux, R uy, R (&feq)[9]) {
    using O = Ieee<R>;
    constexpr R r9 = R(1) / R(9), r36 = R(1) / R(36), r6 = R(1) / R(6);  // RN(1/9), RN(1/36), RN(1/6)
    const R w0 = div_by_rcp(O::mul(R(4), rho), R(9), r9), w1 = div_by_rcp(rho, R(9), r9),
            w5 = div_by_rcp(rho, R(36), r36);
    ux = O::mul(ux, R(3));
    uy = O::mul(uy, R(3));
    const R cu[9] = {R(0), ux, uy, -ux, -uy, O::add(ux, uy), O::add(-ux, uy), O::sub(-ux, uy), O::sub(ux, uy)};
    const R uu = div_by_rcp(O::add(O::mul(ux, ux), O::mul(uy, uy)), R(6), r6);
    feq[0] = O::mul(w0, O::sub(R(1), uu));
#pragma unroll
    for (int i = 1; i < 9; ++i) {
        // 1 - ux is rounded as 1 + (-ux): the same IEEE result
        const R p = O::sub(O::add(O::add(R(1), cu[i]), O::mul(O::mul(cu[i], cu[i]), R(0.5))), uu);
        feq[i] = O::mul(i <= 4 ? w1 : w5, p);
    }
}

template <class R>
__device__ __forceinline__ void bgk_collide_native(R (&f)[9], R omega) {
    using O = Ieee<R>;
    const R rho = O::add(O::add(O::add(f[0], f[1]), O::add(f[2], f[3])),
                         O::add(O::add(f[4], f[5]), O::add(f[6], O::add(f[7], f[8]))));
    R jx = O::sub(f[1], f[3]);
    jx = O::sub(O::sub(O::add(jx, f[5]), f[6]), f[7]);
    jx = O::add(jx, f[8]);
    R jy = O::sub(f[2], f[4]);
    jy = O::sub(O::add(O::add(jy, f[5]), f[6]), f[7]);
    jy = O::sub(jy, f[8]);
    R feq[9];
    const R y = O::rcp(rho);  // RN(1/rho), shared by both quotients
    equilibrium_native(rho, div_by_rcp(jx, rho, y), div_by_rcp(jy, rho, y), feq);
#pragma unroll
    for (int i = 0; i < 9; ++i) f[i] = O::add(f[i], O::mul(omega, O::sub(feq[i], f[i])));
}

// BGK in deviation form, h_i = f_i - w_i (the DEV codecs and the FP32
// kernels), arranged so that the collision conserves momentum by construction.
//
// FP32 rounding of the constants (w_i = 1/9, 1/36; 2/3 = 6 w_1) makes a
// directly evaluated equilibrium carry the momentum j (1 + delta) with
// delta ~ 3e-8, at every node and step: a systematic error that adds up
// (64^2 cavity, omega 1.7, 1000 steps: 4e-6 relative L2 of u against FP64,
// where the rounding of the stored deviations alone gives 8e-8).  Only
// errors in the conserved moments accumulate -- an error in any other moment
// is relaxed away -- so the collision works on the even and odd parts of
// each pair of opposite channels,
//   a_ij = h_i - h_j,  b_ij = h_i + h_j     (pairs 1|3, 2|4, 5|7, 6|8),
// with D = h_0 + sum b, j_x = a13 + a57 - a68, j_y = a24 + a57 + a68,
// rho = 1 + D, u = j / rho:
//   even part (no momentum):  g = w (D - 1.5 j.u + 4.5 (c.j)(c.u)) - b/2
//   odd part of the diagonals: d57 = (j_x + j_y)/12 - a57/2,
//                              d68 = (j_y - j_x)/12 - a68/2
//   odd part of the axes, from the diagonals' (exact algebra of
//   w_i rho 3 c.u with the axis pairs taking the rest of j):
//                              d13 = d68 - d57,  d24 = -(d57 + d68)
//   h_i' = h_i + omega (g +/- d)  (+ for the first channel of the pair).
// The momentum change 2 omega (d13 + d57 - d68, d24 + d57 + d68) is then zero
// whatever the rounding of d57 and d68, and only the final stores round
// momentum.  1/rho enters second-order terms alone (hardware approximation).
// h_0' = D - sum_{i>0} h_i' keeps the node's mass in exact arithmetic of the
// stored values.  In the CPU emulation of this arithmetic the 64^2 cavity is
// at 9e-8 after 1000 and 2000 steps, the storage floor.  Same equilibrium as
// w_i rho (1 + 3 c.u + 4.5 (c.u)^2 - 1.5 u^2) (c/d2q9.h:59-81) in exact
// arithmetic.  REST = false leaves h_0 to the caller, which writes it from
// the rounded stored values.  LOG2K: the values are h 2^LOG2K (FP16 storage
// keeps its deviations scaled by 2^14; a kernel that collides in those units
// skips a scaling per value on decode and encode).  Every operation commutes
// exactly with the power-of-two scale, so the results are bit for bit the
// unscaled ones times 2^LOG2K.  Returns D (in the same units).
template <bool REST = true, int LOG2K = 0>
__device__ __forceinline__ float collide_dev(float (&h)[9], float omega) {
    constexpr float UNIT = 1.f / (float)(1u << LOG2K);
    const float a13 = h[1] - h[3], b13 = h[1] + h[3];
    const float a24 = h[2] - h[4], b24 = h[2] + h[4];
    const float a57 = h[5] - h[7], b57 = h[5] + h[7];
    const float a68 = h[6] - h[8], b68 = h[6] + h[8];
    const float d = (((h[0] + b13) + b24) + b57) + b68;
    const float jx = (a13 + a57) - a68, jy = (a24 + a57) + a68;
    const float inv = recip_approx(fmaf(d, UNIT, 1.f)) * UNIT;
    const float ux = jx * inv, uy = jy * inv;
    const float base = fmaf(-1.5f, fmaf(jx, ux, jy * uy), d);
    const float sx = jx + jy, sy = jy - jx;
    const float g13 = fmaf(-0.5f, b13, (1.f / 9.f) * fmaf(4.5f * jx, ux, base));
    const float g24 = fmaf(-0.5f, b24, (1.f / 9.f) * fmaf(4.5f * jy, uy, base));
    const float g57 = fmaf(-0.5f, b57, (1.f / 36.f) * fmaf(4.5f * sx, ux + uy, base));
    const float g68 = fmaf(-0.5f, b68, (1.f / 36.f) * fmaf(4.5f * sy, uy - ux, base));
    const float d57 = fmaf(sx, 1.f / 12.f, -0.5f * a57);
    const float d68 = fmaf(sy, 1.f / 12.f, -0.5f * a68);
    const float d13 = d68 - d57, d24 = -(d57 + d68);
    h[1] = fmaf(omega, g13 + d13, h[1]);
    h[3] = fmaf(omega, g13 - d13, h[3]);
    h[2] = fmaf(omega, g24 + d24, h[2]);
    h[4] = fmaf(omega, g24 - d24, h[4]);
    h[5] = fmaf(omega, g57 + d57, h[5]);
    h[7] = fmaf(omega, g57 - d57, h[7]);
    h[6] = fmaf(omega, g68 + d68, h[6]);
    h[8] = fmaf(omega, g68 - d68, h[8]);
    if constexpr (REST) {
        float rest = d;
#pragma unroll
        for (int i = 1; i < 9; ++i) rest -= h[i];
        h[0] = rest;
    }
    return d;
}

// The reference lid's Ladd term ((6 w) rho_lid) u0 (cavity_opt1.py:211-212),
// each product rounded on its own, so that the following g +/- term cannot
// be contracted into an FMA: the FP32 and FP64 results then equal the
// reference's rounding of the same expression.
template <class R>
__device__ __forceinline__ R lid_term(R rho_lid, R u0) {
    return Ieee<R>::mul(Ieee<R>::mul(R(6) * R(1.0 / 36.0), rho_lid), u0);
}

// The same term for deviation storage, where the nine summed lid values are
// deviations and rho_lid = 1 + s: c + c s with c = (6 w) u0 rounded once, so
// that the low bits of s are not lost in a rounding of 1 + s (which would
// repeat itself at every lid node and step).
// With the deviations in units of 2^-LOG2K (see collide_dev) the term is
// c s + c 2^LOG2K, the same value in those units.
template <int LOG2K = 0>
__device__ __forceinline__ float lid_term_dev(float s, float u0) {
    const float c = (6.f * (1.f / 36.f)) * u0;
    return fmaf(c, s, c * (float)(1u << LOG2K));
}

// Equilibrium of one node (same formulation as above).
template <class R>
__device__ __forceinline__ void equilibrium1(R rho, R ux, R uy, R (&feq)[9]) {
    const R w0 = rho * R(4.0 / 9.0), w1 = rho * R(1.0 / 9.0), w5 = rho * R(1.0 / 36.0);
    ux *= R(3);
    uy *= R(3);
    const R uu = (ux * ux + uy * uy) * R(1.0 / 6.0);
    const R base = R(1) - uu;
    const R cu5 = ux + uy, cu6 = uy - ux;
    const R hx = R(0.5) * ux * ux, hy = R(0.5) * uy * uy;
    const R h5 = R(0.5) * cu5 * cu5, h6 = R(0.5) * cu6 * cu6;
    feq[0] = w0 * base;
    feq[1] = w1 * (base + ux + hx);
    feq[2] = w1 * (base + uy + hy);
    feq[3] = w1 * (base - ux + hx);
    feq[4] = w1 * (base - uy + hy);
    feq[5] = w5 * (base + cu5 + h5);
    feq[6] = w5 * (base + cu6 + h6);
    feq[7] = w5 * (base - cu5 + h5);
    feq[8] = w5 * (base - cu6 + h6);
}

// The lid's Ladd term from the sum s of the nine lid values of the lid
// density (populations: s = rho_lid; deviations: s = rho_lid - 1).
template <class C>
__device__ __forceinline__ typename C::real lid_from_sum(typename C::real s, typename C::real u0) {
    if constexpr (C::DEV)
        return lid_term_dev(s, u0);
    else
        return lid_term(s, u0);
}

// ---------------------------------------------------------------- conservation
// BGK conserves mass exactly; rounding the nine relaxed values does not, and in
// a slowly varying flow the same rounding repeats step after step and adds up
// (the reference's own float32 path drifts by ~1e-2 in 500 steps of a 48x40
// box with resting walls).  The rest population is therefore written last as
// the node's pre-collision mass minus the eight stored moving populations, so
// that the mass survives the collision up to the rounding of that one value:
//  * FP32: f_0' = f_0 + sum_{i>0} (f_i - f_i'), the relaxed amounts of the
//    moving populations summed as small numbers (exactly zero at rest, so
//    the rest state stays a fixed point; resting-wall drift ~5e-6 instead
//    of ~1e-2, for 16 additions);
//  * 16-bit deviations (half and bfloat16): h_0 = sum_i h_i(before) -
//    sum_{i>0} h_i(stored), the stored values decoded back.  Against FP64
//    (64^2 cavity, moving lid, 1000 steps, CPU emulation of the kernels'
//    arithmetic) the mass drift is then reproduced within 0.5 % (bfloat16)
//    and 0.1 % (half); without the fix bfloat16 misses it by 42 %.
template <int DT>
__device__ __forceinline__ void collide_encode(typename Codec<DT>::real (&f)[9], typename Codec<DT>::real omega,
                                               typename Codec<DT>::raw (&out)[9]) {
    using C = Codec<DT>;
    using real = typename C::real;
    if constexpr (DT == LBGB_F32) {
        // FP32 populations collide in the deviation pair form too: h = f - w
        // (w as stored by the rest state, so the rest state stays a fixed
        // point), collide_dev, f' = h' + w; the populations' own rounding is
        // then the only systematic error left
        real h[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) h[i] = f[i] - wgt<float>(i);
        collide_dev<false>(h, omega);
        real d = 0.f;
#pragma unroll
        for (int i = 1; i < 9; ++i) {
            const real fi = h[i] + wgt<float>(i);
            d += f[i] - fi;
            f[i] = fi;
        }
        f[0] += d;
#pragma unroll
        for (int i = 0; i < 9; ++i) out[i] = f[i];
    } else if constexpr (DT == LBGB_F32DEV) {
        collide_dev(f, omega);
#pragma unroll
        for (int i = 0; i < 9; ++i) out[i] = f[i];
    } else if constexpr (DT == LBGB_F16DEV) {
        // f holds deviations.  The rest population takes the node's scaled
        // mass deviation D S minus what the other eight stored values carry,
        // so the node keeps its mass up to the rounding of h_0 alone.  The
        // pipelined kernel does the same operations.
        real dms = collide_dev<false>(f, omega) * F16_SCALE;
#pragma unroll
        for (int i = 1; i < 9; ++i) {
            out[i] = C::enc_h(f[i]);
            dms = fma16<false>(out[i], F16_MINUS_ONE_BITS, dms);
        }
        out[0] = __half_as_ushort(__float2half_rn(dms));
    } else if constexpr (DT == LBGB_BF16DEV) {
        real dm = collide_dev<false>(f, omega);
#pragma unroll
        for (int i = 1; i < 9; ++i) {
            out[i] = C::enc_h(f[i]);
            dm = sub_stored<DT>(dm, out[i]);
        }
        out[0] = C::enc_h(dm);
    } else {
        bgk_collide(f, omega);
#pragma unroll
        for (int i = 0; i < 9; ++i) out[i] = C::enc(f[i], i);
    }
}

// 16-bit storage with stochastic rounding (see above): the moving deviations
// are rounded stochastically, then the rest population carries the node's
// remaining mass (for both 16-bit codecs) and is rounded stochastically too.
template <int DT>
__device__ __forceinline__ void collide_encode_sr(float (&f)[9], float omega, unsigned short (&out)[9], uint32_t key,
                                                  uint32_t cell) {
    float dm = collide_dev<false>(f, omega);
    const uint32_t base = sr_pair_base(key, cell & ~1u);
    const bool odd = (cell & 1u) != 0u;
    // the cell's own lane of the pair's word, as the packet kernels round it
    auto round1 = [&](float h, int ch) {
        const uint32_t r = sr_channel_bits(base, ch);
        return odd ? (unsigned short)(sr_pack2<DT>(0.f, h, r) >> 16)
                   : (unsigned short)(sr_pack2<DT>(h, 0.f, r) & 0xffffu);
    };
#pragma unroll
    for (int i = 1; i < 9; ++i) {
        out[i] = round1(sr_dev<DT>(f[i]), i);
        dm = sub_stored<DT>(dm, out[i]);
    }
    out[0] = round1(sr_rest<DT>(dm), 0);
}

// ---------------------------------------------------------------- cp.async
// 16-byte global -> shared copies of the issuing thread, grouped; a wait
// returns when at most N of the thread's groups are still in flight (a
// hardware wait on the thread's own copies: nothing to bound).
__device__ __forceinline__ void cp_async16(void *smem_dst, const void *gmem_src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(__cvta_generic_to_global(gmem_src))
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// ---------------------------------------------------------------- host side
void set_error(const char *fmt, ...);
int check_launch(const char *what);

// Current device, clamped into [0, MAX_DEVICES) for per-device host caches
// (kernel attributes and device properties are per device).
constexpr int MAX_DEVICES = 64;
inline int current_device() {
    int d = 0;
    if (cudaGetDevice(&d) != cudaSuccess || d < 0) d = 0;
    return d < MAX_DEVICES ? d : MAX_DEVICES - 1;
}

// One lock for the first-use set-up of the per-device host caches (kernel
// attributes, device properties).  The caches are atomics read without the
// lock; a thread that finds an entry unset takes the lock, sets it up and
// publishes it, so no kernel is launched before its set-up is complete when
// two host threads launch the same variant at once.
inline std::mutex &setup_mutex() {
    static std::mutex m;
    return m;
}

inline bool aligned(const void *p, size_t a) { return (reinterpret_cast<uintptr_t>(p) % a) == 0; }

inline size_t raw_size(int dt) {
    switch (dt) {
    case LBGB_F32:
    case LBGB_F32DEV: return 4;
    case LBGB_F64: return 8;
    case LBGB_F16DEV:
    case LBGB_BF16DEV: return 2;
    default: return 0;
    }
}

}  // namespace lbgb
