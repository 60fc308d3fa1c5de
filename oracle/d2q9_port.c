/*
 * CPU port of the reference D2Q9 BGK hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * Used as (1) a second, compiled checker for the CUDA library and (2) the
 * timed CPU baseline ("port") in bench.py.  The product never links it.
 *
 * Arithmetic follows the reference's native kernel operation by operation:
 *   equilibrium  -> c/d2q9.h:59-81   (ux*=3, uy*=3, uu=(ux^2+uy^2)/6,
 *                                     f_i = w_i rho (1 + cu + cu^2/2 - uu))
 *   collide      -> c/d2q9.h:121-131 (rho = f_i.sum() in the order of
 *                                     Eigen 3.4's unrolled fixed-size
 *                                     reduction, then ux, uy,
 *                                     f += omega (feq - f))
 * Built with -ffp-contract=off: every operation rounds on its own, as in the
 * reference's x86-64 build (no FMA), on x86-64 and aarch64 hosts alike.
 * Streaming follows PyLB/Streaming.py:33-46 (periodic) and
 * simulators/parallel_lid_drive_cavity/cavity_opt1.py:177-245 (half-way
 * bounce-back on four walls, Ladd moving lid, the reference's corner order
 * and its lid density that reads across the periodic seam), written in pull
 * form, out of place.
 *
 * Layout: f[i*nx*ny + k*ny + l], i = channel 0..8, k = x, l = y (l fastest),
 * the layout of a C-contiguous numpy array of shape (9, nx, ny).
 *
 * Threads: OpenMP over rows k; every entry point takes nthreads (<=0: all).
 */
#include <stddef.h>
#include <stdint.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static const int CXv[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
static const int CYv[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
static const int OPPv[9] = {0, 3, 4, 1, 2, 7, 8, 5, 6};
enum { C0 = 0, CE = 1, CN = 2, CW = 3, CS = 4, CNE = 5, CNW = 6, CSW = 7, CSE = 8 };

static void set_threads(int nthreads) {
#ifdef _OPENMP
    omp_set_num_threads(nthreads > 0 ? nthreads : omp_get_num_procs());
#else
    (void)nthreads;
#endif
}

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_num_procs();
#else
    return 1;
#endif
}

#define DEFINE_PORT(T, SUF)                                                          \
static inline void eq1_##SUF(T rho, T ux, T uy, T *o) {                             \
    T w0 = 4 * rho / 9, w1 = rho / 9, w5 = rho / 36;                                 \
    ux *= 3; uy *= 3;                                                                \
    T cu5 = ux + uy, cu6 = -ux + uy, cu7 = -ux - uy, cu8 = ux - uy;                  \
    T uu = (ux * ux + uy * uy) / 6;                                                  \
    o[0] = w0 * (1 - uu);                                                            \
    o[1] = w1 * (1 + ux + ux * ux / 2 - uu);                                         \
    o[2] = w1 * (1 + uy + uy * uy / 2 - uu);                                         \
    o[3] = w1 * (1 - ux + ux * ux / 2 - uu);                                         \
    o[4] = w1 * (1 - uy + uy * uy / 2 - uu);                                         \
    o[5] = w5 * (1 + cu5 + cu5 * cu5 / 2 - uu);                                      \
    o[6] = w5 * (1 + cu6 + cu6 * cu6 / 2 - uu);                                      \
    o[7] = w5 * (1 + cu7 + cu7 * cu7 / 2 - uu);                                      \
    o[8] = w5 * (1 + cu8 + cu8 * cu8 / 2 - uu);                                      \
}                                                                                    \
static inline void collide1_##SUF(T *v, T omega) {                                  \
    /* f_i.sum() of a fixed-size Eigen 3.4 vector: halving split */                  \
    T rho = ((v[0] + v[1]) + (v[2] + v[3])) + ((v[4] + v[5]) + (v[6] + (v[7] + v[8]))); \
    T ux = (v[1] - v[3] + v[5] - v[6] - v[7] + v[8]) / rho;                          \
    T uy = (v[2] - v[4] + v[5] + v[6] - v[7] - v[8]) / rho;                          \
    T e[9];                                                                          \
    eq1_##SUF(rho, ux, uy, e);                                                       \
    for (int i = 0; i < 9; ++i) v[i] += omega * (e[i] - v[i]);                       \
}                                                                                    \
void oracle_equilibrium_##SUF(const T *rho, const T *ux, const T *uy, T *f,          \
                              int64_t n, int64_t cs, int nthreads) {                 \
    set_threads(nthreads);                                                           \
    _Pragma("omp parallel for schedule(static)")                                     \
    for (int64_t c = 0; c < n; ++c) {                                                \
        T e[9];                                                                      \
        eq1_##SUF(rho[c], ux[c], uy[c], e);                                          \
        for (int i = 0; i < 9; ++i) f[i * cs + c] = e[i];                            \
    }                                                                                \
}                                                                                    \
void oracle_collide_##SUF(T *f, int64_t n, int64_t cs, double omega, int nthreads) { \
    set_threads(nthreads);                                                           \
    T om = (T)omega;                                                                 \
    _Pragma("omp parallel for schedule(static)")                                     \
    for (int64_t c = 0; c < n; ++c) {                                                \
        T v[9];                                                                      \
        for (int i = 0; i < 9; ++i) v[i] = f[i * cs + c];                            \
        collide1_##SUF(v, om);                                                       \
        for (int i = 0; i < 9; ++i) f[i * cs + c] = v[i];                            \
    }                                                                                \
}                                                                                    \
void oracle_stream_periodic_##SUF(const T *g, T *f, int nx, int ny, int nthreads) {  \
    set_threads(nthreads);                                                           \
    const int64_t cs = (int64_t)nx * ny;                                             \
    _Pragma("omp parallel for schedule(static)")                                     \
    for (int k = 0; k < nx; ++k)                                                     \
        for (int i = 0; i < 9; ++i) {                                                \
            int ks = ((k - CXv[i]) % nx + nx) % nx;                                  \
            for (int l = 0; l < ny; ++l) {                                           \
                int ls = ((l - CYv[i]) % ny + ny) % ny;                              \
                f[i * cs + (int64_t)k * ny + l] = g[i * cs + (int64_t)ks * ny + ls]; \
            }                                                                        \
        }                                                                            \
}                                                                                    \
/* one node of the cavity pull (rules of cavity_opt1.py:177-245) */                  \
static inline void pull_cavity_##SUF(const T *g, int nx, int ny, int k, int l,       \
                                     T u0, T *v) {                                   \
    const int64_t cs = (int64_t)nx * ny;                                             \
    const int R = nx - 1, Tt = ny - 1;                                               \
    const int64_t at = (int64_t)k * ny + l;                                          \
    for (int i = 0; i < 9; ++i) {                                                    \
        int ks = k - CXv[i], ls = l - CYv[i];                                        \
        if (ks >= 0 && ks < nx && ls >= 0 && ls < ny)                                \
            v[i] = g[i * cs + (int64_t)ks * ny + ls];                                \
        else                                                                         \
            v[i] = g[OPPv[i] * cs + at];                                             \
    }                                                                                \
    if (l == Tt) {                                                                   \
        /* lid density: outgoing NW,N,NE + raw periodic pull of NW,N,NE,W,0,E */     \
        int km = (k + nx - 1) % nx, kp = (k + 1) % nx;                               \
        const int64_t top = (int64_t)k * ny + Tt;                                    \
        T rl = g[CNW * cs + top] + g[CN * cs + top] + g[CNE * cs + top]              \
             + g[CNW * cs + (int64_t)kp * ny + Tt - 1]                               \
             + g[CN * cs + (int64_t)k * ny + Tt - 1]                                 \
             + g[CNE * cs + (int64_t)km * ny + Tt - 1]                               \
             + g[CW * cs + (int64_t)kp * ny + Tt]                                    \
             + g[C0 * cs + top]                                                      \
             + g[CE * cs + (int64_t)km * ny + Tt];                                   \
        T w6 = (T)6 * (T)(1.0 / 36.0);                                               \
        if (k != 0) v[CSE] = g[CNW * cs + top] + w6 * rl * u0;                       \
        if (k != R) v[CSW] = g[CNE * cs + top] - w6 * rl * u0;                       \
    }                                                                                \
}                                                                                    \
void oracle_stream_bb_##SUF(const T *g, T *f, int nx, int ny, double u0,             \
                            int nthreads) {                                          \
    set_threads(nthreads);                                                           \
    const int64_t cs = (int64_t)nx * ny;                                             \
    T u = (T)u0;                                                                     \
    _Pragma("omp parallel for schedule(static)")                                     \
    for (int k = 0; k < nx; ++k)                                                     \
        for (int l = 0; l < ny; ++l) {                                               \
            T v[9];                                                                  \
            pull_cavity_##SUF(g, nx, ny, k, l, u, v);                                \
            for (int i = 0; i < 9; ++i) f[i * cs + (int64_t)k * ny + l] = v[i];      \
        }                                                                            \
}                                                                                    \
/* nsteps of the reference's cavity step, each a stream+bounce-back pass and a      \
 * collide pass as in cavity_opt2.py:276-277; a and b are swapped every step and   \
 * the return value tells which buffer holds the result (0: a, 1: b). */            \
int oracle_cavity_run_##SUF(T *a, T *b, int nx, int ny, double omega, double u0,     \
                            int nsteps, int nthreads) {                              \
    T *src = a, *dst = b;                                                            \
    const int64_t n = (int64_t)nx * ny;                                              \
    for (int s = 0; s < nsteps; ++s) {                                               \
        oracle_stream_bb_##SUF(src, dst, nx, ny, u0, nthreads);                      \
        oracle_collide_##SUF(dst, n, n, omega, nthreads);                            \
        T *t = src; src = dst; dst = t;                                              \
    }                                                                                \
    return src == a ? 0 : 1;                                                         \
}                                                                                    \
int oracle_periodic_run_##SUF(T *a, T *b, int nx, int ny, double omega,              \
                              int nsteps, int nthreads) {                            \
    T *src = a, *dst = b;                                                            \
    const int64_t n = (int64_t)nx * ny;                                              \
    for (int s = 0; s < nsteps; ++s) {                                               \
        oracle_stream_periodic_##SUF(src, dst, nx, ny, nthreads);                    \
        oracle_collide_##SUF(dst, n, n, omega, nthreads);                            \
        T *t = src; src = dst; dst = t;                                              \
    }                                                                                \
    return src == a ? 0 : 1;                                                         \
}

DEFINE_PORT(double, f64)
DEFINE_PORT(float, f32)

/* Sum over all populations and first moments, in double (mass, x and y momentum). */
void oracle_mass_momentum_f64(const double *f, int64_t n, double *out) {
    double m = 0, px = 0, py = 0;
    for (int i = 0; i < 9; ++i)
        for (int64_t c = 0; c < n; ++c) {
            double v = f[i * n + c];
            m += v; px += CXv[i] * v; py += CYv[i] * v;
        }
    out[0] = m; out[1] = px; out[2] = py;
}
