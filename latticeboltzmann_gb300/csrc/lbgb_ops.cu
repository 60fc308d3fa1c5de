// Node-local operators of liblbgb (equilibrium, collision, macroscopic fields,
// storage conversion), the deterministic mass/momentum reduction, and the
// library's error state.
#include <stdarg.h>
#include <stdio.h>

#include <mutex>

#include "lbgb_common.cuh"

namespace lbgb {

// ---------------------------------------------------------------- errors
static thread_local char g_err[512] = "";

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

int check_launch(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("%s: %s", what, cudaGetErrorString(e));
        return LBGB_ECUDA;
    }
    return LBGB_OK;
}

static int grid_for(int64_t items, int threads) {
    int64_t b = (items + threads - 1) / threads;
    if (b > (1 << 20)) b = 1 << 20;  // grid-stride beyond this
    return (int)(b < 1 ? 1 : b);
}

// ---------------------------------------------------------------- equilibrium
// The native kernel's operations in its order (d2q9_equilibriumn,
// c/d2q9.h:98-108): bit for bit the reference's float and double results.
template <class T>
__global__ void k_equilibrium(const T *__restrict__ rho, const T *__restrict__ ux, const T *__restrict__ uy,
                              T *__restrict__ f, int64_t n, int64_t cs) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
        T feq[9];
        equilibrium_native<T>(rho[c], ux[c], uy[c], feq);
#pragma unroll
        for (int i = 0; i < 9; ++i) f[i * cs + c] = feq[i];
    }
}

// ------------------------------------------------------- Chapman-Enskog start
// f_i = f_i^eq(rho, u) - (3 w_i rho / omega) Q_iab d_a u_b,  Q_iab = c_ia c_ib - delta_ab / 3
// (first-order non-equilibrium part of the Chapman-Enskog expansion, c_s^2 = 1/3),
// or the post-collision state f^eq + (1 - omega) f^neq that a time step leaves.
// Velocity gradients: central differences; for the cavity the boundary nodes
// take the quadratic through the wall value (half a cell out: 0, or the lid
// velocity) and the next two nodes:  du/dx(0) = -4/3 u_wall + u(0) + u(1)/3.
template <class T>
__device__ __forceinline__ T grad1(const T *__restrict__ u, int64_t at, int64_t stride, int i, int n, bool periodic,
                                   T wall_lo, T wall_hi) {
    if (periodic || n < 2) {
        if (n < 2) return T(0);
        const int64_t lo = i == 0 ? at + (int64_t)(n - 1) * stride : at - stride;
        const int64_t hi = i == n - 1 ? at - (int64_t)(n - 1) * stride : at + stride;
        return T(0.5) * (u[hi] - u[lo]);
    }
    if (i == 0) return -T(4.0 / 3.0) * wall_lo + u[at] + u[at + stride] * T(1.0 / 3.0);
    if (i == n - 1) return T(4.0 / 3.0) * wall_hi - u[at] - u[at - stride] * T(1.0 / 3.0);
    return T(0.5) * (u[at + stride] - u[at - stride]);
}

template <class T>
__global__ void k_chapman_enskog(const T *__restrict__ rho, const T *__restrict__ ux, const T *__restrict__ uy,
                                 T *__restrict__ f, int nx, int ny, T omega, T u0, int boundary, T neq_scale) {
    const int64_t n = (int64_t)nx * ny;
    const bool per = boundary == LBGB_PERIODIC;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
        const int k = (int)(c / ny), l = (int)(c - (int64_t)k * ny);
        // lid at l = ny-1 moves with (u0, 0); every other wall rests
        const T dxux = grad1<T>(ux, c, ny, k, nx, per, T(0), T(0));
        const T dxuy = grad1<T>(uy, c, ny, k, nx, per, T(0), T(0));
        const T dyux = grad1<T>(ux, c, 1, l, ny, per, T(0), u0);
        const T dyuy = grad1<T>(uy, c, 1, l, ny, per, T(0), T(0));
        T feq[9];
        equilibrium1<T>(rho[c], ux[c], uy[c], feq);
        const T pre = neq_scale * T(3) * rho[c] / omega;
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            const T ex = T(cx(i)), ey = T(cy(i));
            const T q = (ex * ex - T(1.0 / 3.0)) * dxux + ex * ey * (dxuy + dyux) + (ey * ey - T(1.0 / 3.0)) * dyuy;
            f[i * n + c] = feq[i] - pre * wgt<T>(i) * q;
        }
    }
}

// ---------------------------------------------------------------- collide
// One thread relaxes V consecutive cells; vector access when the channel
// stride and the pointer allow it, else element by element.  NATIVE (FP32
// and FP64 only): the reference native kernel's arithmetic, operation by
// operation (bgk_collide_native); otherwise the solver's collision with its
// mass-preserving store (collide_encode).
// Resident blocks per SM the register allocation must allow: the FP32
// native-order collision of four cells per thread fits 80 registers without
// spilling (three blocks of 256 threads per SM); the others keep the
// compiler's choice (a bound of three makes them spill).
template <int DT, int V, bool NATIVE>
constexpr int collide_min_blocks() { return (DT == LBGB_F32 && V == 4 && NATIVE) ? 3 : 1; }

template <int DT, int V, bool NATIVE>
__global__ void __launch_bounds__(256, collide_min_blocks<DT, V, NATIVE>())
k_collide(typename Codec<DT>::raw *__restrict__ f, int64_t n, int64_t cs, typename Codec<DT>::real omega) {
    using C = Codec<DT>;
    using raw = typename C::raw;
    using real = typename C::real;
    const int64_t groups = (n + V - 1) / V;
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < groups;
         g += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c0 = g * V;
        const int cnt = (int)((n - c0) < V ? (n - c0) : V);
        real v[9][V];
        if (cnt == V) {
#pragma unroll
            for (int i = 0; i < 9; ++i) {
                raw r[V];
                ldv<raw, V>(f + i * cs + c0, r);
#pragma unroll
                for (int j = 0; j < V; ++j) v[i][j] = C::dec(r[j], i);
            }
        } else {
#pragma unroll
            for (int i = 0; i < 9; ++i)
#pragma unroll
                for (int j = 0; j < V; ++j) v[i][j] = j < cnt ? C::dec(f[i * cs + c0 + j], i) : real(1.0 / 9.0);
        }
        raw out[9][V];
#pragma unroll
        for (int j = 0; j < V; ++j) {
            real x[9];
            raw r[9];
#pragma unroll
            for (int i = 0; i < 9; ++i) x[i] = v[i][j];
            if constexpr (NATIVE) {
                bgk_collide_native(x, omega);
#pragma unroll
                for (int i = 0; i < 9; ++i) r[i] = x[i];
            } else {
                collide_encode<DT>(x, omega, r);
            }
#pragma unroll
            for (int i = 0; i < 9; ++i) out[i][j] = r[i];
        }
        if (cnt == V) {
#pragma unroll
            for (int i = 0; i < 9; ++i) stv<raw, V>(f + i * cs + c0, out[i]);
        } else {
            // constant indices only (a loop bound of cnt would put out[][] in local memory)
#pragma unroll
            for (int i = 0; i < 9; ++i)
#pragma unroll
                for (int j = 0; j < V; ++j)
                    if (j < cnt) f[i * cs + c0 + j] = out[i][j];
        }
    }
}

template <int DT, bool NATIVE>
static int launch_collide(void *f, int64_t n, int64_t cs, double omega, cudaStream_t s) {
    using C = Codec<DT>;
    constexpr int VW = 16 / sizeof(typename C::raw);
    if (cs % VW == 0 && aligned(f, 16)) {
        k_collide<DT, VW, NATIVE><<<grid_for((n + VW - 1) / VW, 256), 256, 0, s>>>(
            static_cast<typename C::raw *>(f), n, cs, (typename C::real)omega);
    } else {
        k_collide<DT, 1, NATIVE><<<grid_for(n, 256), 256, 0, s>>>(static_cast<typename C::raw *>(f), n, cs,
                                                                  (typename C::real)omega);
    }
    return check_launch("k_collide");
}

// ---------------------------------------------------------------- macroscopic
template <int DT>
__global__ void k_macroscopic(const typename Codec<DT>::raw *__restrict__ f, typename Codec<DT>::real *rho,
                              typename Codec<DT>::real *ux, typename Codec<DT>::real *uy, int64_t n, int64_t cs) {
    using C = Codec<DT>;
    using real = typename C::real;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
        real v[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) v[i] = C::dec(f[i * cs + c], i);
        const real r = node_density<DT>(v);
        // same expressions as the reference's diagnostics (cavity_opt1.py:154-156)
        const real jx = v[1] - v[3] + v[5] - v[6] - v[7] + v[8];
        const real jy = v[2] - v[4] + v[5] + v[6] - v[7] - v[8];
        if (rho) rho[c] = r;
        if (ux) ux[c] = jx / r;
        if (uy) uy[c] = jy / r;
    }
}

// ------------------------------------------------------ row spectrum amplitude
// The decay diagnostic of simulators/simple_flows/shear_wave_decay.py:155-158:
// 2/ny * max_k |DFT_k(ux[row, :])|, in FP64 (direct transform, one block).
constexpr int SPEC_MAX_NY = 4096;

template <int DT>
__global__ void __launch_bounds__(256) k_row_fft_amplitude(const typename Codec<DT>::raw *__restrict__ f, int nx,
                                                           int ny, int row, double *__restrict__ out) {
    using C = Codec<DT>;
    __shared__ double u[SPEC_MAX_NY];
    __shared__ double red[256];
    const int64_t cs = (int64_t)nx * ny;
    for (int l = threadIdx.x; l < ny; l += blockDim.x) {
        const int64_t c = (int64_t)row * ny + l;
        double v[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) v[i] = C::decd(f[i * cs + c], i);
        double r = v[0];
#pragma unroll
        for (int i = 1; i < 9; ++i) r += v[i];
        u[l] = (v[1] - v[3] + v[5] - v[6] - v[7] + v[8]) / r;
    }
    __syncthreads();
    double best = 0.0;
    for (int k = threadIdx.x; k < ny; k += blockDim.x) {
        double re = 0.0, im = 0.0;
        int64_t ph = 0;  // k * l mod ny, kept exact
        for (int l = 0; l < ny; ++l) {
            double sv, cv;
            sincospi(2.0 * (double)ph / (double)ny, &sv, &cv);
            re += u[l] * cv;
            im -= u[l] * sv;
            ph += k;
            if (ph >= ny) ph -= ny;
        }
        best = fmax(best, sqrt(re * re + im * im));
    }
    red[threadIdx.x] = best;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = 2.0 / ny * red[0];
}

// ---------------------------------------------------------------- channel walls
// Dry wall rows y = 0 and y = ny-1 of the simple-flow scripts (convention B):
// after a push stream, what entered a wall row is reflected into the adjacent
// fluid row; the top wall moves with uw (SW, SE gain -uw/6, +uw/6).  One
// thread per column, in the scripts' statement order (bottom, then top), so
// ny = 2 and 3 give the same result as the sequential numpy code.
template <class T>
__global__ void k_wall_bounce_back(T *__restrict__ f, int nx, int ny, T uw6, int k0, int k1, int clear) {
    const int64_t cs = (int64_t)nx * ny;
    const int t = ny - 1;
    for (int k = k0 + blockIdx.x * blockDim.x + threadIdx.x; k < k1; k += gridDim.x * blockDim.x) {
        T *col = f + (int64_t)k * ny;
        col[2 * cs + 1] = col[4 * cs];
        col[5 * cs + 1] = col[7 * cs];
        col[6 * cs + 1] = col[8 * cs];
        if (clear) col[4 * cs] = col[7 * cs] = col[8 * cs] = T(0);
        col[4 * cs + t - 1] = col[2 * cs + t];
        col[7 * cs + t - 1] = col[5 * cs + t] - uw6;
        col[8 * cs + t - 1] = col[6 * cs + t] + uw6;
        if (clear) col[2 * cs + t] = col[5 * cs + t] = col[6 * cs + t] = T(0);
    }
}

// Solid nodes of any shape (a mask), link-wise: after a push stream, the
// population f_i found at a solid node x came from y = x - c_i; if y is fluid
// it returns there as f_opp(i)(y).  Each (y, opp(i)) has one source, solid
// nodes are only read and fluid nodes only written, so one thread per node
// needs no ordering.
template <class T>
__global__ void k_solid_bounce_back(T *__restrict__ f, const unsigned char *__restrict__ solid, int nx, int ny,
                                    int periodic) {
    const int64_t n = (int64_t)nx * ny;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
        if (!solid[c]) continue;
        const int k = (int)(c / ny), l = (int)(c - (int64_t)k * ny);
#pragma unroll
        for (int i = 1; i < 9; ++i) {
            int ks = k - cx(i), ls = l - cy(i);
            if (periodic) {
                ks = ks < 0 ? ks + nx : (ks >= nx ? ks - nx : ks);
                ls = ls < 0 ? ls + ny : (ls >= ny ? ls - ny : ls);
            } else if (ks < 0 || ks >= nx || ls < 0 || ls >= ny) {
                continue;
            }
            const int64_t y = (int64_t)ks * ny + ls;
            if (!solid[y]) f[opp(i) * n + y] = f[i * n + c];
        }
    }
}

// Pressure-periodic ghost columns: x = 0 takes the equilibrium at rho_in with
// the velocity of column nx-2 plus that column's non-equilibrium part; x =
// nx-1 the same with rho_out and column 1.  One thread per row; every input
// is read before either ghost is written.
template <class T>
__global__ void k_pressure_periodic(T *__restrict__ f, int nx, int ny, T rho_in, T rho_out) {
    const int64_t cs = (int64_t)nx * ny;
    for (int l = blockIdx.x * blockDim.x + threadIdx.x; l < ny; l += gridDim.x * blockDim.x) {
        T a[9], b[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            a[i] = f[i * cs + (int64_t)(nx - 2) * ny + l];
            b[i] = f[i * cs + (int64_t)1 * ny + l];
        }
        T ra = a[0], rb = b[0];
#pragma unroll
        for (int i = 1; i < 9; ++i) {
            ra += a[i];
            rb += b[i];
        }
        const T uxa = (a[1] - a[3] + a[5] - a[6] - a[7] + a[8]) / ra, uya = (a[2] - a[4] + a[5] + a[6] - a[7] - a[8]) / ra;
        const T uxb = (b[1] - b[3] + b[5] - b[6] - b[7] + b[8]) / rb, uyb = (b[2] - b[4] + b[5] + b[6] - b[7] - b[8]) / rb;
        T ea[9], eb[9], ein[9], eout[9];
        equilibrium1<T>(ra, uxa, uya, ea);
        equilibrium1<T>(rb, uxb, uyb, eb);
        equilibrium1<T>(rho_in, uxa, uya, ein);
        equilibrium1<T>(rho_out, uxb, uyb, eout);
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            f[i * cs + l] = ein[i] + (a[i] - ea[i]);
            f[i * cs + (int64_t)(nx - 1) * ny + l] = eout[i] + (b[i] - eb[i]);
        }
    }
}

// ---------------------------------------------------------------- convert
template <int SD, int DD>
__global__ void k_convert(const typename Codec<SD>::raw *__restrict__ src, int64_t ss,
                          typename Codec<DD>::raw *__restrict__ dst, int64_t ds, int64_t n) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            dst[i * ds + c] = Codec<DD>::encd(Codec<SD>::decd(src[i * ss + c], i), i);
        }
    }
}

template <int SD>
static int launch_convert_to(const void *src, int64_t ss, void *dst, int dd, int64_t ds, int64_t n, cudaStream_t s) {
    const int g = grid_for(n, 256);
    const auto *a = static_cast<const typename Codec<SD>::raw *>(src);
    switch (dd) {
    case LBGB_F32: k_convert<SD, LBGB_F32><<<g, 256, 0, s>>>(a, ss, static_cast<float *>(dst), ds, n); break;
    case LBGB_F64: k_convert<SD, LBGB_F64><<<g, 256, 0, s>>>(a, ss, static_cast<double *>(dst), ds, n); break;
    case LBGB_F16DEV:
        k_convert<SD, LBGB_F16DEV><<<g, 256, 0, s>>>(a, ss, static_cast<unsigned short *>(dst), ds, n);
        break;
    case LBGB_BF16DEV:
        k_convert<SD, LBGB_BF16DEV><<<g, 256, 0, s>>>(a, ss, static_cast<unsigned short *>(dst), ds, n);
        break;
    case LBGB_F32DEV: k_convert<SD, LBGB_F32DEV><<<g, 256, 0, s>>>(a, ss, static_cast<float *>(dst), ds, n); break;
    default: set_error("lbgb_convert: unsupported destination storage code %d", dd); return LBGB_EDTYPE;
    }
    return check_launch("k_convert");
}

// ---------------------------------------------------------------- mass/momentum
// Two passes with a fixed grid: pass 1 writes one (mass, px, py) partial per
// block into the workspace, pass 2 sums the partials in block order.  The
// grid size does not depend on the device, so the sum is reproducible.
constexpr int RED_BLOCKS = 1024;
constexpr int RED_THREADS = 256;

template <int DT>
__global__ void __launch_bounds__(RED_THREADS)
k_mass_momentum_partial(const typename Codec<DT>::raw *__restrict__ f, int64_t n, int64_t cs, double *partial) {
    using C = Codec<DT>;
    double m = 0.0, px = 0.0, py = 0.0;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
        double v[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) v[i] = C::decd(f[i * cs + c], i);
        double r = v[0];
#pragma unroll
        for (int i = 1; i < 9; ++i) r += v[i];
        m += r;
        px += v[1] - v[3] + v[5] - v[6] - v[7] + v[8];
        py += v[2] - v[4] + v[5] + v[6] - v[7] - v[8];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        m += __shfl_down_sync(0xffffffffu, m, o);
        px += __shfl_down_sync(0xffffffffu, px, o);
        py += __shfl_down_sync(0xffffffffu, py, o);
    }
    __shared__ double sm[3][RED_THREADS / 32];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        sm[0][w] = m;
        sm[1][w] = px;
        sm[2][w] = py;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double acc = 0.0;
        for (int i = 0; i < RED_THREADS / 32; ++i) acc += sm[threadIdx.x][i];
        partial[blockIdx.x * 3 + threadIdx.x] = acc;
    }
}

__global__ void __launch_bounds__(RED_THREADS) k_sum_partials(const double *partial, int nblocks, double *out) {
    // thread t sums partials t, t+256, ... then a fixed-order tree
    __shared__ double sm[3][RED_THREADS];
    for (int q = 0; q < 3; ++q) {
        double acc = 0.0;
        for (int b = threadIdx.x; b < nblocks; b += RED_THREADS) acc += partial[b * 3 + q];
        sm[q][threadIdx.x] = acc;
    }
    __syncthreads();
    for (int s = RED_THREADS / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s)
            for (int q = 0; q < 3; ++q) sm[q][threadIdx.x] += sm[q][threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x < 3) out[threadIdx.x] = sm[threadIdx.x][0];
}

static int check_cells(const void *f, int64_t n, int64_t cs, int dtype, const char *what) {
    if (raw_size(dtype) == 0) {
        set_error("%s: unsupported storage code %d", what, dtype);
        return LBGB_EDTYPE;
    }
    if (n < 0 || cs < n) {
        set_error("%s: need 0 <= n <= chan_stride (n=%lld, chan_stride=%lld)", what, (long long)n, (long long)cs);
        return LBGB_EINVAL;
    }
    if (n > 0 && !f) {
        set_error("%s: null population pointer", what);
        return LBGB_EINVAL;
    }
    if (!aligned(f, raw_size(dtype))) {
        set_error("%s: population pointer must be aligned to the element size", what);
        return LBGB_EINVAL;
    }
    return LBGB_OK;
}

}  // namespace lbgb

using namespace lbgb;

extern "C" int lbgb_version(void) { return 1 * 10000 + 0 * 100 + 0; }

extern "C" int lbgb_last_error(char *buf, size_t len) {
    const size_t n = strlen(g_err);
    if (buf && len) {
        const size_t m = n < len - 1 ? n : len - 1;
        memcpy(buf, g_err, m);
        buf[m] = 0;
    }
    return (int)n;
}

extern "C" int lbgb_equilibrium(const void *rho, const void *ux, const void *uy, void *f, int64_t n,
                                int64_t chan_stride, int dtype, void *stream) {
    int rc = check_cells(f, n, chan_stride, dtype, "lbgb_equilibrium");
    if (rc) return rc;
    if (n == 0) return LBGB_OK;
    if (!rho || !ux || !uy) {
        set_error("lbgb_equilibrium: null field pointer");
        return LBGB_EINVAL;
    }
    cudaStream_t s = (cudaStream_t)stream;
    if (dtype == LBGB_F32) {
        k_equilibrium<float><<<grid_for(n, 256), 256, 0, s>>>((const float *)rho, (const float *)ux,
                                                              (const float *)uy, (float *)f, n, chan_stride);
    } else if (dtype == LBGB_F64) {
        k_equilibrium<double><<<grid_for(n, 256), 256, 0, s>>>((const double *)rho, (const double *)ux,
                                                               (const double *)uy, (double *)f, n, chan_stride);
    } else {
        set_error("lbgb_equilibrium: storage code %d not supported (F32 or F64)", dtype);
        return LBGB_EDTYPE;
    }
    return check_launch("k_equilibrium");
}

extern "C" int lbgb_chapman_enskog(const void *rho, const void *ux, const void *uy, void *f, int nx, int ny,
                                   double omega, double u0, int boundary, int post_collision, int dtype,
                                   void *stream) {
    if (!rho || !ux || !uy || !f || nx <= 0 || ny <= 0 || !(omega > 0.0)) {
        set_error("lbgb_chapman_enskog: bad arguments (nx=%d ny=%d omega=%g)", nx, ny, omega);
        return LBGB_EINVAL;
    }
    if (boundary != LBGB_PERIODIC && boundary != LBGB_CAVITY && boundary != LBGB_CAVITY_LADD) {
        set_error("lbgb_chapman_enskog: unknown boundary code %d", boundary);
        return LBGB_EINVAL;
    }
    const int64_t n = (int64_t)nx * ny;
    cudaStream_t s = (cudaStream_t)stream;
    const double lid = boundary == LBGB_PERIODIC ? 0.0 : u0;
    const double scale = post_collision ? 1.0 - omega : 1.0;
    if (dtype == LBGB_F32) {
        k_chapman_enskog<float><<<grid_for(n, 256), 256, 0, s>>>((const float *)rho, (const float *)ux,
                                                                 (const float *)uy, (float *)f, nx, ny, (float)omega,
                                                                 (float)lid, boundary, (float)scale);
    } else if (dtype == LBGB_F64) {
        k_chapman_enskog<double><<<grid_for(n, 256), 256, 0, s>>>((const double *)rho, (const double *)ux,
                                                                  (const double *)uy, (double *)f, nx, ny, omega,
                                                                  lid, boundary, scale);
    } else {
        set_error("lbgb_chapman_enskog: storage code %d not supported (F32 or F64)", dtype);
        return LBGB_EDTYPE;
    }
    return check_launch("k_chapman_enskog");
}

extern "C" int lbgb_row_fft_amplitude(const void *f, int nx, int ny, int row, int dtype, double *out_dev,
                                      void *stream) {
    if (!f || !out_dev || nx <= 0 || ny <= 0 || ny > SPEC_MAX_NY || row < 0 || row >= nx) {
        set_error("lbgb_row_fft_amplitude: bad arguments (nx=%d ny=%d row=%d; ny <= %d)", nx, ny, row, SPEC_MAX_NY);
        return LBGB_EINVAL;
    }
    cudaStream_t s = (cudaStream_t)stream;
    switch (dtype) {
    case LBGB_F32: k_row_fft_amplitude<LBGB_F32><<<1, 256, 0, s>>>((const float *)f, nx, ny, row, out_dev); break;
    case LBGB_F64: k_row_fft_amplitude<LBGB_F64><<<1, 256, 0, s>>>((const double *)f, nx, ny, row, out_dev); break;
    case LBGB_F16DEV:
        k_row_fft_amplitude<LBGB_F16DEV><<<1, 256, 0, s>>>((const unsigned short *)f, nx, ny, row, out_dev);
        break;
    case LBGB_BF16DEV:
        k_row_fft_amplitude<LBGB_BF16DEV><<<1, 256, 0, s>>>((const unsigned short *)f, nx, ny, row, out_dev);
        break;
    case LBGB_F32DEV: k_row_fft_amplitude<LBGB_F32DEV><<<1, 256, 0, s>>>((const float *)f, nx, ny, row, out_dev); break;
    default: set_error("lbgb_row_fft_amplitude: unsupported storage code %d", dtype); return LBGB_EDTYPE;
    }
    return check_launch("k_row_fft_amplitude");
}

extern "C" int lbgb_wall_bounce_back(void *f, int nx, int ny, double uw, int interior, int clear, int dtype,
                                     void *stream) {
    if (!f || nx <= 0 || ny < 2 || (interior && nx < 3)) {
        set_error("lbgb_wall_bounce_back: need ny >= 2 (and nx >= 3 for interior columns), got %d x %d", nx, ny);
        return LBGB_EINVAL;
    }
    const int k0 = interior ? 1 : 0, k1 = interior ? nx - 1 : nx;
    const int g = (k1 - k0 + 255) / 256;
    cudaStream_t s = (cudaStream_t)stream;
    const double uw6 = 1.0 / 6.0 * uw;
    if (dtype == LBGB_F32)
        k_wall_bounce_back<float><<<g, 256, 0, s>>>((float *)f, nx, ny, (float)uw6, k0, k1, clear);
    else if (dtype == LBGB_F64)
        k_wall_bounce_back<double><<<g, 256, 0, s>>>((double *)f, nx, ny, uw6, k0, k1, clear);
    else {
        set_error("lbgb_wall_bounce_back: storage code %d not supported (F32 or F64)", dtype);
        return LBGB_EDTYPE;
    }
    return check_launch("k_wall_bounce_back");
}

extern "C" int lbgb_solid_bounce_back(void *f, const void *solid, int nx, int ny, int periodic, int dtype,
                                      void *stream) {
    if (!f || !solid || nx <= 0 || ny <= 0) {
        set_error("lbgb_solid_bounce_back: bad arguments (nx=%d ny=%d)", nx, ny);
        return LBGB_EINVAL;
    }
    const int64_t n = (int64_t)nx * ny;
    cudaStream_t s = (cudaStream_t)stream;
    const auto *m = static_cast<const unsigned char *>(solid);
    if (dtype == LBGB_F32)
        k_solid_bounce_back<float><<<grid_for(n, 256), 256, 0, s>>>((float *)f, m, nx, ny, periodic);
    else if (dtype == LBGB_F64)
        k_solid_bounce_back<double><<<grid_for(n, 256), 256, 0, s>>>((double *)f, m, nx, ny, periodic);
    else {
        set_error("lbgb_solid_bounce_back: storage code %d not supported (F32 or F64)", dtype);
        return LBGB_EDTYPE;
    }
    return check_launch("k_solid_bounce_back");
}

extern "C" int lbgb_pressure_periodic(void *f, int nx, int ny, double rho_in, double rho_out, int dtype,
                                      void *stream) {
    if (!f || nx < 2 || ny <= 0) {
        set_error("lbgb_pressure_periodic: need nx >= 2 and ny >= 1, got %d x %d", nx, ny);
        return LBGB_EINVAL;
    }
    const int g = (ny + 255) / 256;
    cudaStream_t s = (cudaStream_t)stream;
    if (dtype == LBGB_F32)
        k_pressure_periodic<float><<<g, 256, 0, s>>>((float *)f, nx, ny, (float)rho_in, (float)rho_out);
    else if (dtype == LBGB_F64)
        k_pressure_periodic<double><<<g, 256, 0, s>>>((double *)f, nx, ny, rho_in, rho_out);
    else {
        set_error("lbgb_pressure_periodic: storage code %d not supported (F32 or F64)", dtype);
        return LBGB_EDTYPE;
    }
    return check_launch("k_pressure_periodic");
}

extern "C" int lbgb_copy_rows(void *dst, const void *src, int nx, int ny, int k_begin, int k_end, int dtype,
                              void *stream) {
    if (!dst || !src || nx <= 0 || ny <= 0 || k_begin < 0 || k_end > nx || k_begin > k_end) {
        set_error("lbgb_copy_rows: bad arguments (nx=%d ny=%d rows [%d, %d))", nx, ny, k_begin, k_end);
        return LBGB_EINVAL;
    }
    const size_t es = raw_size(dtype);
    if (es == 0) {
        set_error("lbgb_copy_rows: unsupported storage code %d", dtype);
        return LBGB_EDTYPE;
    }
    if (k_begin == k_end) return LBGB_OK;
    const size_t pitch = (size_t)nx * ny * es, row = (size_t)ny * es, off = (size_t)k_begin * row;
    // nine channel planes, rows [k_begin, k_end) of each: one strided copy
    cudaError_t e = cudaMemcpy2DAsync(static_cast<char *>(dst) + off, pitch, static_cast<const char *>(src) + off, pitch,
                                      (size_t)(k_end - k_begin) * row, 9, cudaMemcpyDefault, (cudaStream_t)stream);
    if (e != cudaSuccess) {
        set_error("lbgb_copy_rows: %s", cudaGetErrorString(e));
        return LBGB_ECUDA;
    }
    return LBGB_OK;
}

extern "C" int lbgb_collide_ex(void *f, int64_t n, int64_t chan_stride, int dtype, double omega, int flags,
                               void *stream) {
    int rc = check_cells(f, n, chan_stride, dtype, "lbgb_collide");
    if (rc) return rc;
    if (flags & ~LBGB_COLLIDE_KEEP_MASS) {
        set_error("lbgb_collide_ex: unknown flags 0x%x", flags);
        return LBGB_EINVAL;
    }
    if (n == 0) return LBGB_OK;
    cudaStream_t s = (cudaStream_t)stream;
    const bool keep = (flags & LBGB_COLLIDE_KEEP_MASS) != 0;
    switch (dtype) {
    case LBGB_F32:
        return keep ? launch_collide<LBGB_F32, false>(f, n, chan_stride, omega, s)
                    : launch_collide<LBGB_F32, true>(f, n, chan_stride, omega, s);
    case LBGB_F64:
        return keep ? launch_collide<LBGB_F64, false>(f, n, chan_stride, omega, s)
                    : launch_collide<LBGB_F64, true>(f, n, chan_stride, omega, s);
    // the deviation storages always keep each node's mass through the stored values
    case LBGB_F16DEV: return launch_collide<LBGB_F16DEV, false>(f, n, chan_stride, omega, s);
    case LBGB_BF16DEV: return launch_collide<LBGB_BF16DEV, false>(f, n, chan_stride, omega, s);
    case LBGB_F32DEV: return launch_collide<LBGB_F32DEV, false>(f, n, chan_stride, omega, s);
    }
    return LBGB_EDTYPE;
}

extern "C" int lbgb_collide(void *f, int64_t n, int64_t chan_stride, int dtype, double omega, void *stream) {
    return lbgb_collide_ex(f, n, chan_stride, dtype, omega, 0, stream);
}

extern "C" int lbgb_macroscopic(const void *f, void *rho, void *ux, void *uy, int64_t n, int64_t chan_stride,
                                int dtype, void *stream) {
    int rc = check_cells(f, n, chan_stride, dtype, "lbgb_macroscopic");
    if (rc) return rc;
    if (n == 0) return LBGB_OK;
    cudaStream_t s = (cudaStream_t)stream;
    const int g = grid_for(n, 256);
    switch (dtype) {
    case LBGB_F32:
        k_macroscopic<LBGB_F32><<<g, 256, 0, s>>>((const float *)f, (float *)rho, (float *)ux, (float *)uy, n,
                                                  chan_stride);
        break;
    case LBGB_F64:
        k_macroscopic<LBGB_F64><<<g, 256, 0, s>>>((const double *)f, (double *)rho, (double *)ux, (double *)uy, n,
                                                  chan_stride);
        break;
    case LBGB_F16DEV:
        k_macroscopic<LBGB_F16DEV><<<g, 256, 0, s>>>((const unsigned short *)f, (float *)rho, (float *)ux,
                                                     (float *)uy, n, chan_stride);
        break;
    case LBGB_BF16DEV:
        k_macroscopic<LBGB_BF16DEV><<<g, 256, 0, s>>>((const unsigned short *)f, (float *)rho, (float *)ux,
                                                      (float *)uy, n, chan_stride);
        break;
    case LBGB_F32DEV:
        k_macroscopic<LBGB_F32DEV><<<g, 256, 0, s>>>((const float *)f, (float *)rho, (float *)ux, (float *)uy, n,
                                                     chan_stride);
        break;
    }
    return check_launch("k_macroscopic");
}

extern "C" size_t lbgb_mass_momentum_workspace_bytes(void) { return (size_t)RED_BLOCKS * 3 * sizeof(double); }

extern "C" int lbgb_mass_momentum(const void *f, int64_t n, int64_t chan_stride, int dtype, double *out_dev,
                                  void *workspace, size_t workspace_bytes, void *stream) {
    int rc = check_cells(f, n, chan_stride, dtype, "lbgb_mass_momentum");
    if (rc) return rc;
    if (!out_dev) {
        set_error("lbgb_mass_momentum: null output pointer");
        return LBGB_EINVAL;
    }
    if (!workspace || workspace_bytes < lbgb_mass_momentum_workspace_bytes() || !aligned(workspace, 8)) {
        set_error("lbgb_mass_momentum: workspace needs %zu bytes, 8-byte aligned (got %zu)",
                  lbgb_mass_momentum_workspace_bytes(), workspace_bytes);
        return LBGB_EWORKSPACE;
    }
    cudaStream_t s = (cudaStream_t)stream;
    double *partial = static_cast<double *>(workspace);
    switch (dtype) {
    case LBGB_F32:
        k_mass_momentum_partial<LBGB_F32><<<RED_BLOCKS, RED_THREADS, 0, s>>>((const float *)f, n, chan_stride, partial);
        break;
    case LBGB_F64:
        k_mass_momentum_partial<LBGB_F64><<<RED_BLOCKS, RED_THREADS, 0, s>>>((const double *)f, n, chan_stride,
                                                                             partial);
        break;
    case LBGB_F16DEV:
        k_mass_momentum_partial<LBGB_F16DEV><<<RED_BLOCKS, RED_THREADS, 0, s>>>((const unsigned short *)f, n,
                                                                                chan_stride, partial);
        break;
    case LBGB_BF16DEV:
        k_mass_momentum_partial<LBGB_BF16DEV><<<RED_BLOCKS, RED_THREADS, 0, s>>>((const unsigned short *)f, n,
                                                                                 chan_stride, partial);
        break;
    case LBGB_F32DEV:
        k_mass_momentum_partial<LBGB_F32DEV><<<RED_BLOCKS, RED_THREADS, 0, s>>>((const float *)f, n, chan_stride,
                                                                                partial);
        break;
    }
    rc = check_launch("k_mass_momentum_partial");
    if (rc) return rc;
    k_sum_partials<<<1, RED_THREADS, 0, s>>>(partial, RED_BLOCKS, out_dev);
    return check_launch("k_sum_partials");
}

extern "C" int lbgb_convert(const void *src, int src_dtype, int64_t src_stride, void *dst, int dst_dtype,
                            int64_t dst_stride, int64_t n, void *stream) {
    int rc = check_cells(src, n, src_stride, src_dtype, "lbgb_convert");
    if (rc) return rc;
    rc = check_cells(dst, n, dst_stride, dst_dtype, "lbgb_convert");
    if (rc) return rc;
    if (n == 0) return LBGB_OK;
    cudaStream_t s = (cudaStream_t)stream;
    switch (src_dtype) {
    case LBGB_F32: return launch_convert_to<LBGB_F32>(src, src_stride, dst, dst_dtype, dst_stride, n, s);
    case LBGB_F64: return launch_convert_to<LBGB_F64>(src, src_stride, dst, dst_dtype, dst_stride, n, s);
    case LBGB_F16DEV: return launch_convert_to<LBGB_F16DEV>(src, src_stride, dst, dst_dtype, dst_stride, n, s);
    case LBGB_BF16DEV: return launch_convert_to<LBGB_BF16DEV>(src, src_stride, dst, dst_dtype, dst_stride, n, s);
    case LBGB_F32DEV: return launch_convert_to<LBGB_F32DEV>(src, src_stride, dst, dst_dtype, dst_stride, n, s);
    }
    return LBGB_EDTYPE;
}

// ---------------------------------------------------------------- allocation-free reduction
// lbgb_mass_momentum_noalloc is for callers that are not allowed to allocate
// device memory at all -- for example a simulation code embedded in a larger
// application whose memory manager owns the whole GPU, or a time loop where a
// device allocation (which can synchronise the device and can fail when memory
// is short) is forbidden between steps -- and so cannot provide the workspace
// that lbgb_mass_momentum asks for.  It runs the same two kernels, with the
// per-block partial sums kept in the file-scope array below instead of a
// caller's workspace.
//
// Limits and sharing:
//  * one partial per 4096 cells, at most LBGB_NOALLOC_MAX_CELLS cells (the
//    array holds 65536 partials = 1.5 MiB; every GPU that loads this library
//    holds it until the process exits);
//  * every call uses the same array: each block overwrites its own partial
//    before the second kernel reads it, so nothing has to start at zero, but
//    calls whose kernels overlap on the GPU (different streams without
//    ordering) race on the array and give wrong sums.
constexpr int NOALLOC_CELLS_PER_BLOCK = RED_THREADS * 16;
constexpr int NOALLOC_MAX_BLOCKS = (int)(LBGB_NOALLOC_MAX_CELLS / NOALLOC_CELLS_PER_BLOCK);
static __device__ __align__(256) double g_noalloc_partials[NOALLOC_MAX_BLOCKS * 3];

// Device address of the array, looked up once per device with that device
// current.  A host-side use of the symbol itself would be a host stand-in,
// not a device address, and must never be handed to a kernel.
static double *noalloc_partials(int *rc) {
    constexpr int MAX_DEV = 64;
    static double *ptr[MAX_DEV] = {};
    static std::mutex mu;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= MAX_DEV) {
        set_error("lbgb_mass_momentum_noalloc: no usable current device (%s)",
                  e != cudaSuccess ? cudaGetErrorString(e) : "device index out of range");
        *rc = LBGB_ECUDA;
        return nullptr;
    }
    std::lock_guard<std::mutex> lock(mu);
    if (!ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_partials);
        if (e != cudaSuccess || !p) {
            set_error("lbgb_mass_momentum_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
            *rc = LBGB_ECUDA;
            return nullptr;
        }
        ptr[dev] = static_cast<double *>(p);
    }
    *rc = LBGB_OK;
    return ptr[dev];
}

extern "C" int lbgb_mass_momentum_noalloc(const void *f, int64_t n, int64_t chan_stride, int dtype, double *out_dev,
                                         void *stream) {
    int rc = check_cells(f, n, chan_stride, dtype, "lbgb_mass_momentum_noalloc");
    if (rc) return rc;
    if (!out_dev) {
        set_error("lbgb_mass_momentum_noalloc: null output pointer");
        return LBGB_EINVAL;
    }
    if (n > LBGB_NOALLOC_MAX_CELLS) {
        set_error("lbgb_mass_momentum_noalloc: %lld cells exceed the built-in scratch limit of %lld cells; "
                  "use lbgb_mass_momentum with a workspace",
                  (long long)n, (long long)LBGB_NOALLOC_MAX_CELLS);
        return LBGB_EINVAL;
    }
    double *partial = noalloc_partials(&rc);
    if (!partial) return rc;
    const int nblocks = n > 0 ? (int)((n + NOALLOC_CELLS_PER_BLOCK - 1) / NOALLOC_CELLS_PER_BLOCK) : 1;
    cudaStream_t s = (cudaStream_t)stream;
    switch (dtype) {
    case LBGB_F32:
        k_mass_momentum_partial<LBGB_F32><<<nblocks, RED_THREADS, 0, s>>>((const float *)f, n, chan_stride, partial);
        break;
    case LBGB_F64:
        k_mass_momentum_partial<LBGB_F64><<<nblocks, RED_THREADS, 0, s>>>((const double *)f, n, chan_stride,
                                                                          partial);
        break;
    case LBGB_F16DEV:
        k_mass_momentum_partial<LBGB_F16DEV><<<nblocks, RED_THREADS, 0, s>>>((const unsigned short *)f, n,
                                                                             chan_stride, partial);
        break;
    case LBGB_BF16DEV:
        k_mass_momentum_partial<LBGB_BF16DEV><<<nblocks, RED_THREADS, 0, s>>>((const unsigned short *)f, n,
                                                                              chan_stride, partial);
        break;
    case LBGB_F32DEV:
        k_mass_momentum_partial<LBGB_F32DEV><<<nblocks, RED_THREADS, 0, s>>>((const float *)f, n, chan_stride,
                                                                             partial);
        break;
    default: set_error("lbgb_mass_momentum_noalloc: unsupported storage code %d", dtype); return LBGB_EDTYPE;
    }
    rc = check_launch("k_mass_momentum_partial (no-alloc)");
    if (rc) return rc;
    k_sum_partials<<<1, RED_THREADS, 0, s>>>(partial, nblocks, out_dev);
    return check_launch("k_sum_partials (no-alloc)");
}
