// Element-wise and mode-mixing kernels of the Fourier-neural-operator
// surrogate (the GEMMs are in lbgb_gemm.cu).  Activations are channel-major,
// (C, B*H*W): channel c's values for all samples and grid points are
// contiguous, so a pointwise layer is one GEMM over B*H*W columns.
#include "lbgb_act.cuh"
#include "lbgb_common.cuh"

namespace lbgb {

__global__ void k_to_bf16(const float *__restrict__ x, __nv_bfloat16 *__restrict__ y, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        y[i] = __float2bfloat16_rn(x[i]);
}

// z[c, j] += bias[c] (+ extra[c, j]); act: 0 identity, 1 GELU -> v (fp32 and bf16).
// Grid (column blocks, channel): no per-element index division.
__global__ void k_bias_act(float *__restrict__ z, const float *__restrict__ bias, const float *__restrict__ extra,
                           float *__restrict__ v, __nv_bfloat16 *__restrict__ vb, long long cols, int act) {
    const int c = blockIdx.y;
    const float b = bias ? bias[c] : 0.f;
    const long long base = (long long)c * cols;
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < cols; j += (long long)gridDim.x * blockDim.x) {
        const long long i = base + j;
        float x = z[i] + b + (extra ? extra[i] : 0.f);
        z[i] = x;
        const float y = act ? gelu_f(x) : x;
        if (v) v[i] = y;
        if (vb) vb[i] = __float2bfloat16_rn(y);
    }
}

// dz = dy * gelu'(z), also as bf16
__global__ void k_gelu_back(const float *__restrict__ dy, const float *__restrict__ z, float *__restrict__ dz,
                            __nv_bfloat16 *__restrict__ dzb, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float g = dy[i] * gelu_df(z[i]);
        dz[i] = g;
        if (dzb) dzb[i] = __float2bfloat16_rn(g);
    }
}

// Four consecutive elements per thread: 16-byte loads and stores, 8-byte
// stores of the BF16 copies.  The launchers take these when every row is a
// whole number of float4 and every pointer is aligned; the per-element
// arithmetic is that of the scalar kernels above, so results are identical.
__device__ __forceinline__ uint2 pack_bf16x4(float4 y) {
    const __nv_bfloat162 lo = __floats2bfloat162_rn(y.x, y.y), hi = __floats2bfloat162_rn(y.z, y.w);
    uint2 r;
    memcpy(&r.x, &lo, 4);
    memcpy(&r.y, &hi, 4);
    return r;
}

__global__ void k_to_bf16_4(const float4 *__restrict__ x, uint2 *__restrict__ y, long long n4) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n4; i += (long long)gridDim.x * blockDim.x)
        y[i] = pack_bf16x4(x[i]);
}

__global__ void k_bias_act4(float4 *__restrict__ z, const float *__restrict__ bias, const float4 *__restrict__ extra,
                            float4 *__restrict__ v, uint2 *__restrict__ vb, long long cols4, int act) {
    const int c = blockIdx.y;
    const float b = bias ? bias[c] : 0.f;
    const long long base = (long long)c * cols4;
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < cols4;
         j += (long long)gridDim.x * blockDim.x) {
        const long long i = base + j;
        float4 x = z[i];
        const float4 e = extra ? extra[i] : make_float4(0.f, 0.f, 0.f, 0.f);
        x.x = x.x + b + e.x;
        x.y = x.y + b + e.y;
        x.z = x.z + b + e.z;
        x.w = x.w + b + e.w;
        z[i] = x;
        const float4 y = act ? make_float4(gelu_f(x.x), gelu_f(x.y), gelu_f(x.z), gelu_f(x.w)) : x;
        if (v) v[i] = y;
        if (vb) vb[i] = pack_bf16x4(y);
    }
}

__global__ void k_gelu_back4(const float4 *__restrict__ dy, const float4 *__restrict__ z, float4 *__restrict__ dz,
                             uint2 *__restrict__ dzb, long long n4) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n4; i += (long long)gridDim.x * blockDim.x) {
        const float4 d = dy[i], x = z[i];
        const float4 g = make_float4(d.x * gelu_df(x.x), d.y * gelu_df(x.y), d.z * gelu_df(x.z), d.w * gelu_df(x.w));
        dz[i] = g;
        if (dzb) dzb[i] = pack_bf16x4(g);
    }
}

// db[c] = sum_j dy[c, j]: block (chunk, c) sums one of ROWSUM_CHUNKS slices
// of row c into part[c][chunk]; k_row_sum_finish adds the slices in order
// (deterministic, and every SM busy however few channels there are).
constexpr int ROWSUM_CHUNKS = 64;

// V = 4: the row is read as float4 (cols a multiple of 4, dy aligned)
template <int V>
__global__ void __launch_bounds__(256) k_row_sum(const float *__restrict__ dy, float *__restrict__ part, long long cols) {
    const int c = blockIdx.y, chunk = blockIdx.x;
    const long long units = cols / V;
    const long long len = (units + ROWSUM_CHUNKS - 1) / ROWSUM_CHUNKS;
    const long long j0 = chunk * len, j1 = j0 + len < units ? j0 + len : units;
    float acc = 0.f;
    for (long long j = j0 + threadIdx.x; j < j1; j += blockDim.x) {
        if constexpr (V == 4) {
            const float4 x = reinterpret_cast<const float4 *>(dy + c * cols)[j];
            acc += x.x;
            acc += x.y;
            acc += x.z;
            acc += x.w;
        } else {
            acc += dy[c * cols + j];
        }
    }
    __shared__ float sm[256];
    sm[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sm[threadIdx.x] += sm[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[c * ROWSUM_CHUNKS + chunk] = sm[0];
}

__global__ void k_row_sum_finish(const float *__restrict__ part, float *__restrict__ db, int channels) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= channels) return;
    float s = 0.f;
    for (int k = 0; k < ROWSUM_CHUNKS; ++k) s += part[c * ROWSUM_CHUNKS + k];
    db[c] = s;
}

// Complex mixing per Fourier mode, on the layouts of the factorised DFT GEMMs
// (q kept ky values, mk kept kx values):
//   P  (C, B, 2mk, 2q) FP32: P[j][n], j < mk: Re of the W-transform at kx = j,
//      j >= mk: its Im at kx = j - mk; n < q: times cos(ky_n), n >= q: sin(ky_{n-q})
//   so x = xr + i xi with xr = P[kx][y] + P[mk+kx][q+y], xi = P[mk+kx][y] - P[kx][q+y];
//   R  (C, O, q, mk) BF16 (real, imaginary parts);
//   Ym (O, B, 2q, 2mk) BF16, the right operand of the inverse transform along H:
//      rows y: [yr | yi], rows q+y: [-yi | yr], with y = sum_c x R (complex).
__device__ __forceinline__ void mode_x(const float *__restrict__ Pcb, int y, int kx, int q, int mk, float &xr,
                                       float &xi) {
    const int q2 = 2 * q;
    xr = Pcb[kx * q2 + y] + Pcb[(mk + kx) * q2 + q + y];
    xi = Pcb[(mk + kx) * q2 + y] - Pcb[kx * q2 + q + y];
}
__device__ __forceinline__ void mode_dy(const float *__restrict__ D, int y, int kx, int q, int mk, float &dyr,
                                        float &dyi) {
    const int m2 = 2 * mk;
    dyr = D[y * m2 + kx] + D[(q + y) * m2 + mk + kx];
    dyi = D[y * m2 + mk + kx] - D[(q + y) * m2 + kx];
}

__global__ void k_mix_fwd(const float *__restrict__ P, const __nv_bfloat16 *__restrict__ Rr,
                          const __nv_bfloat16 *__restrict__ Ri, __nv_bfloat16 *__restrict__ Ym, int C, int O, int B,
                          int q, int mk) {
    const int Q = q * mk;
    const long long n = (long long)O * B * Q;
    const long long pcb = 4LL * mk * q;  // P elements per (c, b)
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const int mode = (int)(t % Q), y = mode / mk, kx = mode % mk;
        const int b = (int)((t / Q) % B);
        const int o = (int)(t / ((long long)Q * B));
        float ar = 0.f, ai = 0.f;
        for (int c = 0; c < C; ++c) {
            float xr, xi;
            mode_x(P + ((long long)c * B + b) * pcb, y, kx, q, mk, xr, xi);
            const long long r = ((long long)c * O + o) * Q + mode;
            const float rr = __bfloat162float(Rr[r]), ri = __bfloat162float(Ri[r]);
            ar += xr * rr - xi * ri;
            ai += xr * ri + xi * rr;
        }
        __nv_bfloat16 *Y = Ym + ((long long)o * B + b) * pcb;
        const int m2 = 2 * mk;
        Y[y * m2 + kx] = __float2bfloat16_rn(ar);
        Y[y * m2 + mk + kx] = __float2bfloat16_rn(ai);
        Y[(q + y) * m2 + kx] = __float2bfloat16_rn(-ai);
        Y[(q + y) * m2 + mk + kx] = __float2bfloat16_rn(ar);
    }
}

// Gradient with respect to the inputs: dYm (O, B, 2q, 2mk) FP32 -> dP (C, B, 2mk, 2q) BF16
__global__ void k_mix_bwd_x(const float *__restrict__ dYm, const __nv_bfloat16 *__restrict__ Rr,
                            const __nv_bfloat16 *__restrict__ Ri, __nv_bfloat16 *__restrict__ dP, int C, int O, int B,
                            int q, int mk) {
    const int Q = q * mk;
    const long long n = (long long)C * B * Q;
    const long long pcb = 4LL * mk * q;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const int mode = (int)(t % Q), y = mode / mk, kx = mode % mk;
        const int b = (int)((t / Q) % B);
        const int c = (int)(t / ((long long)Q * B));
        float ar = 0.f, ai = 0.f;
        for (int o = 0; o < O; ++o) {
            float gr, gi;
            mode_dy(dYm + ((long long)o * B + b) * pcb, y, kx, q, mk, gr, gi);
            const long long r = ((long long)c * O + o) * Q + mode;
            const float rr = __bfloat162float(Rr[r]), ri = __bfloat162float(Ri[r]);
            ar += gr * rr + gi * ri;
            ai += -gr * ri + gi * rr;
        }
        __nv_bfloat16 *D = dP + ((long long)c * B + b) * pcb;
        const int q2 = 2 * q;
        D[kx * q2 + y] = __float2bfloat16_rn(ar);
        D[(mk + kx) * q2 + q + y] = __float2bfloat16_rn(ar);
        D[(mk + kx) * q2 + y] = __float2bfloat16_rn(ai);
        D[kx * q2 + q + y] = __float2bfloat16_rn(-ai);
    }
}

// Gradient with respect to the weights: dR (C, O, q, mk) FP32, summed over the batch
__global__ void k_mix_bwd_r(const float *__restrict__ dYm, const float *__restrict__ P, float *__restrict__ dRr,
                            float *__restrict__ dRi, int C, int O, int B, int q, int mk) {
    const int Q = q * mk;
    const long long n = (long long)C * O * Q;
    const long long pcb = 4LL * mk * q;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const int mode = (int)(t % Q), y = mode / mk, kx = mode % mk;
        const int o = (int)((t / Q) % O);
        const int c = (int)(t / ((long long)Q * O));
        float ar = 0.f, ai = 0.f;
        for (int b = 0; b < B; ++b) {
            float gr, gi, xr, xi;
            mode_dy(dYm + ((long long)o * B + b) * pcb, y, kx, q, mk, gr, gi);
            mode_x(P + ((long long)c * B + b) * pcb, y, kx, q, mk, xr, xi);
            ar += gr * xr + gi * xi;
            ai += -gr * xi + gi * xr;
        }
        dRr[t] = ar;
        dRi[t] = ai;
    }
}

// mean squared error: partial sums per block into part[], and d = 2 (y - t) / n
__global__ void __launch_bounds__(256) k_mse(const float *__restrict__ y, const float *__restrict__ t,
                                             float *__restrict__ d, double *__restrict__ part, long long n) {
    double acc = 0.0;
    const float s = 2.f / (float)n;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float e = y[i] - t[i];
        acc += (double)e * e;
        d[i] = s * e;
    }
    __shared__ double sm[256];
    sm[threadIdx.x] = acc;
    __syncthreads();
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
        if (threadIdx.x < k) sm[threadIdx.x] += sm[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sm[0];
}

// Weighted squared error: element i lies in plane i / plane of (cout, B) planes
// of H*W elements each, and plane p carries the weight w[p].  Loss partials
// sum w_p e^2, d = 2 w_p e / n.
__global__ void __launch_bounds__(256) k_mse_weighted(const float *__restrict__ y, const float *__restrict__ t,
                                                      const float *__restrict__ w, long long plane,
                                                      float *__restrict__ d, double *__restrict__ part, long long n) {
    double acc = 0.0;
    const float s = 2.f / (float)n;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float e = y[i] - t[i];
        const float wp = w[i / plane];
        acc += (double)wp * e * e;
        d[i] = s * wp * e;
    }
    __shared__ double sm[256];
    sm[threadIdx.x] = acc;
    __syncthreads();
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
        if (threadIdx.x < k) sm[threadIdx.x] += sm[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sm[0];
}

// Adam on FP32 master weights, refreshing their BF16 copies
__global__ void k_adam(float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m, float *__restrict__ v,
                       __nv_bfloat16 *__restrict__ wb, long long n, float lr, float b1, float b2, float eps, float c1,
                       float c2, float wd) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float gi = g[i] + wd * w[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        w[i] = wi;
        if (wb) wb[i] = __float2bfloat16_rn(wi);
    }
}

// out[i] = beta * out[i] + sum_s parts[s * n + i]   (split-K partial sums).
// A block of 32 x SUM_GROUPS threads takes 32 consecutive outputs: thread
// (x, y) adds the splits s = y, y + SUM_GROUPS, ... (loads coalesced over x),
// then the group sums are added in the fixed order y = 0, 1, ...  (One
// thread per output walking all S splits left the few hundred threads of a
// weight gradient waiting on S dependent additions.)
constexpr int SUM_GROUPS = 8;
__global__ void __launch_bounds__(32 * SUM_GROUPS)
k_sum_splits(const float *__restrict__ parts, float *__restrict__ out, int S, long long n, float beta) {
    __shared__ float part[SUM_GROUPS][33];
    const long long i = blockIdx.x * 32ll + threadIdx.x;
    float acc = 0.f;
    if (i < n) {
#pragma unroll 4
        for (int s = threadIdx.y; s < S; s += SUM_GROUPS) acc += parts[(long long)s * n + i];
    }
    part[threadIdx.y][threadIdx.x] = acc;
    __syncthreads();
    if (threadIdx.y == 0 && i < n) {
        float t = beta == 0.f ? 0.f : beta * out[i];
#pragma unroll
        for (int y = 0; y < SUM_GROUPS; ++y) t += part[y][threadIdx.x];
        out[i] = t;
    }
}

static int blocks_for(long long n) {
    long long b = (n + 255) / 256;
    if (b > 8192) b = 8192;
    return (int)(b < 1 ? 1 : b);
}

}  // namespace lbgb

using namespace lbgb;

extern "C" int lbgb_fno_to_bf16(const float *x, void *y, long long n, void *stream) {
    if (n <= 0) return LBGB_OK;
    if (n % 4 == 0 && aligned(x, 16) && aligned(y, 8)) {
        k_to_bf16_4<<<blocks_for(n / 4), 256, 0, (cudaStream_t)stream>>>(reinterpret_cast<const float4 *>(x),
                                                                           static_cast<uint2 *>(y), n / 4);
        return check_launch("k_to_bf16_4");
    }
    k_to_bf16<<<blocks_for(n), 256, 0, (cudaStream_t)stream>>>(x, static_cast<__nv_bfloat16 *>(y), n);
    return check_launch("k_to_bf16");
}

extern "C" int lbgb_fno_bias_act(float *z, const float *bias, const float *extra, float *v, void *vb, int channels,
                                 long long cols, int act, void *stream) {
    const long long n = (long long)channels * cols;
    if (n <= 0) return LBGB_OK;
    if (channels > 65535) {
        set_error("lbgb_fno_bias_act: at most 65535 channels");
        return LBGB_EINVAL;
    }
    const bool v4 = cols % 4 == 0 && aligned(z, 16) && (!extra || aligned(extra, 16)) && (!v || aligned(v, 16)) &&
                    (!vb || aligned(vb, 8));
    const long long units = v4 ? cols / 4 : cols;
    long long per = (units + 255) / 256;
    const long long cap = (8192 + channels - 1) / channels;  // ~8192 blocks in all
    const int gx = (int)(per < cap ? (per < 1 ? 1 : per) : cap);
    if (v4) {
        k_bias_act4<<<dim3(gx, channels), 256, 0, (cudaStream_t)stream>>>(
            reinterpret_cast<float4 *>(z), bias, reinterpret_cast<const float4 *>(extra), reinterpret_cast<float4 *>(v),
            static_cast<uint2 *>(vb), units, act);
        return check_launch("k_bias_act4");
    }
    k_bias_act<<<dim3(gx, channels), 256, 0, (cudaStream_t)stream>>>(z, bias, extra, v, static_cast<__nv_bfloat16 *>(vb),
                                                                     cols, act);
    return check_launch("k_bias_act");
}

extern "C" int lbgb_fno_gelu_back(const float *dy, const float *z, float *dz, void *dzb, long long n, void *stream) {
    if (n <= 0) return LBGB_OK;
    if (n % 4 == 0 && aligned(dy, 16) && aligned(z, 16) && aligned(dz, 16) && (!dzb || aligned(dzb, 8))) {
        k_gelu_back4<<<blocks_for(n / 4), 256, 0, (cudaStream_t)stream>>>(
            reinterpret_cast<const float4 *>(dy), reinterpret_cast<const float4 *>(z), reinterpret_cast<float4 *>(dz),
            static_cast<uint2 *>(dzb), n / 4);
        return check_launch("k_gelu_back4");
    }
    k_gelu_back<<<blocks_for(n), 256, 0, (cudaStream_t)stream>>>(dy, z, dz, static_cast<__nv_bfloat16 *>(dzb), n);
    return check_launch("k_gelu_back");
}

extern "C" int lbgb_fno_row_sum(const float *dy, float *db, float *partials, int channels, long long cols,
                                void *stream) {
    if (channels <= 0 || channels > 65535) {
        set_error("lbgb_fno_row_sum: 1 <= channels <= 65535");
        return LBGB_EINVAL;
    }
    cudaStream_t s = (cudaStream_t)stream;
    if (cols % 4 == 0 && aligned(dy, 16))
        k_row_sum<4><<<dim3(ROWSUM_CHUNKS, channels), 256, 0, s>>>(dy, partials, cols);
    else
        k_row_sum<1><<<dim3(ROWSUM_CHUNKS, channels), 256, 0, s>>>(dy, partials, cols);
    int rc = check_launch("k_row_sum");
    if (rc) return rc;
    k_row_sum_finish<<<(channels + 127) / 128, 128, 0, s>>>(partials, db, channels);
    return check_launch("k_row_sum_finish");
}

extern "C" int lbgb_fno_mix(const float *P, const void *Rr, const void *Ri, void *Ym, int C, int O, int B, int q,
                            int mk, void *stream) {
    const long long n = (long long)O * B * q * mk;
    if (n <= 0 || C <= 0) return LBGB_OK;
    k_mix_fwd<<<blocks_for(n), 256, 0, (cudaStream_t)stream>>>(P, static_cast<const __nv_bfloat16 *>(Rr),
                                                               static_cast<const __nv_bfloat16 *>(Ri),
                                                               static_cast<__nv_bfloat16 *>(Ym), C, O, B, q, mk);
    return check_launch("k_mix_fwd");
}

extern "C" int lbgb_fno_mix_back(const float *dYm, const float *P, const void *Rr, const void *Ri, void *dP,
                                 float *dRr, float *dRi, int C, int O, int B, int q, int mk, void *stream) {
    if (C <= 0 || O <= 0 || B <= 0 || q <= 0 || mk <= 0) return LBGB_OK;
    cudaStream_t s = (cudaStream_t)stream;
    k_mix_bwd_x<<<blocks_for((long long)C * B * q * mk), 256, 0, s>>>(
        dYm, static_cast<const __nv_bfloat16 *>(Rr), static_cast<const __nv_bfloat16 *>(Ri),
        static_cast<__nv_bfloat16 *>(dP), C, O, B, q, mk);
    int rc = check_launch("k_mix_bwd_x");
    if (rc) return rc;
    k_mix_bwd_r<<<blocks_for((long long)C * O * q * mk), 256, 0, s>>>(dYm, P, dRr, dRi, C, O, B, q, mk);
    return check_launch("k_mix_bwd_r");
}

extern "C" int lbgb_fno_mse(const float *y, const float *t, float *d, double *partials, int nparts, long long n,
                            void *stream) {
    if (nparts <= 0 || nparts > 8192) {
        set_error("lbgb_fno_mse: 1 <= nparts <= 8192");
        return LBGB_EINVAL;
    }
    k_mse<<<nparts, 256, 0, (cudaStream_t)stream>>>(y, t, d, partials, n);
    return check_launch("k_mse");
}

extern "C" int lbgb_fno_mse_weighted(const float *y, const float *t, const float *w, long long plane, float *d,
                                     double *partials, int nparts, long long n, void *stream) {
    if (nparts <= 0 || nparts > 8192) {
        set_error("lbgb_fno_mse_weighted: 1 <= nparts <= 8192");
        return LBGB_EINVAL;
    }
    if (plane <= 0 || n % plane != 0 || !w) {
        set_error("lbgb_fno_mse_weighted: n must be a positive multiple of the plane size and w given");
        return LBGB_EINVAL;
    }
    k_mse_weighted<<<nparts, 256, 0, (cudaStream_t)stream>>>(y, t, w, plane, d, partials, n);
    return check_launch("k_mse_weighted");
}

extern "C" int lbgb_fno_adam(float *w, const float *g, float *m, float *v, void *wb, long long n, float lr, float b1,
                             float b2, float eps, int step, float weight_decay, void *stream) {
    if (n <= 0) return LBGB_OK;
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    k_adam<<<blocks_for(n), 256, 0, (cudaStream_t)stream>>>(w, g, m, v, static_cast<__nv_bfloat16 *>(wb), n, lr, b1,
                                                            b2, eps, c1, c2, weight_decay);
    return check_launch("k_adam");
}

extern "C" int lbgb_fno_sum_splits(const float *parts, float *out, int S, long long n, float beta, void *stream) {
    if (n <= 0) return LBGB_OK;
    if (S <= 0) {
        set_error("lbgb_fno_sum_splits: S must be positive");
        return LBGB_EINVAL;
    }
    const long long blocks = (n + 31) / 32;
    if (blocks > 2147483647ll) {
        set_error("lbgb_fno_sum_splits: too many outputs");
        return LBGB_EINVAL;
    }
    k_sum_splits<<<(unsigned)blocks, dim3(32, SUM_GROUPS), 0, (cudaStream_t)stream>>>(parts, out, S, n, beta);
    return check_launch("k_sum_splits");
}
