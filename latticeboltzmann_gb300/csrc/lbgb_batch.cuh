// Many independent lattices of uneven size advanced by one launch per step.
//
// The populations of all instances live in one buffer, instance b at element
// offset `offset` as a (9, nx, ny) array.  The work is a packed queue of tasks
// (instance, first row, first column of a 32*V-cell row segment): one warp
// takes one task and advances `rows_per_task` consecutive rows of that
// segment with the same per-segment code as the single-lattice register
// kernel (step_segment), so instances of any size share the GPU at the
// granularity of a warp.  Instances whose rows hold whole 16-byte vectors use
// V = 16 / sizeof(element) cells per lane, the others one cell per lane
// (the table's `vec` field, warp-uniform).  The CTAs are persistent: the grid
// is sized by the caller (autotuned) and strides over the queue.
//
// Table entries and tasks are checked in the kernel against the buffer size
// and the instance count; an entry that does not fit is skipped, never
// dereferenced.
#pragma once

namespace lbgb {

struct BatchInstanceDev {
    long long offset;
    int nx, ny;
    double omega, u0;
    int vec;
    unsigned int cell_base;
};
static_assert(sizeof(BatchInstanceDev) == sizeof(lbgb_batch_instance), "instance table layout");

template <int DT, int BC, int VW>
__global__ void __launch_bounds__(256)
k_batch_step(const typename Codec<DT>::raw *__restrict__ src, typename Codec<DT>::raw *__restrict__ dst,
             long long total_elems, const BatchInstanceDev *__restrict__ inst, int n_inst,
             const int4 *__restrict__ tasks, long long n_tasks, int rows_per_task) {
    using real = typename Codec<DT>::real;
    const int lane = threadIdx.x & 31;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long t = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < n_tasks; t += nwarps) {
        const int4 tk = tasks[t];
        if (tk.x < 0 || tk.x >= n_inst) continue;
        const BatchInstanceDev in = inst[tk.x];
        const long long need = 9ll * in.nx * in.ny;
        if (in.nx <= 0 || in.ny <= 0 || in.offset < 0 || in.offset + need > total_elems) continue;
        if (BC != LBGB_PERIODIC && (in.nx < 2 || in.ny < 2)) continue;
        if (tk.y < 0 || tk.z < 0 || tk.z >= in.ny) continue;
        const bool wide = in.vec == VW && in.ny % VW == 0 && tk.z % VW == 0 && in.offset % VW == 0;
        for (int r = 0; r < rows_per_task; ++r) {
            const int k = tk.y + r;
            if (k >= in.nx) break;
            if (wide)
                step_segment<DT, BC, true, VW>(src + in.offset, dst + in.offset, in.nx, in.ny, k, tk.z + lane * VW,
                                               lane, (real)in.omega, (real)in.u0, nullptr, 0u, in.cell_base);
            else
                step_segment<DT, BC, true, 1>(src + in.offset, dst + in.offset, in.nx, in.ny, k, tk.z + lane, lane,
                                              (real)in.omega, (real)in.u0, nullptr, 0u, in.cell_base);
        }
    }
}

// Flat tasks: lane j of a task owns cell c0 + 32*r + j of the flattened
// (nx*ny) grid of one instance (rows back to back, every lane busy however
// short the rows are) and pulls its nine populations with direct loads --
// consecutive lanes read consecutive addresses, and the one-cell shifts of
// neighbouring lanes meet in L1/L2, so DRAM still sees each value once.
template <class C, int BC>
__device__ __forceinline__ void pull_cell(const typename C::raw *__restrict__ src, int nx, int ny, int k, int l,
                                          typename C::real u0, typename C::real (&v)[9]) {
    using real = typename C::real;
    const long long n = (long long)nx * ny;
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        int ks = k - cx(i), ls = l - cy(i);
        if (BC == LBGB_PERIODIC) {
            ks = ks < 0 ? ks + nx : (ks >= nx ? ks - nx : ks);
            ls = ls < 0 ? ls + ny : (ls >= ny ? ls - ny : ls);
            v[i] = C::dec(ld1(src + i * n + (long long)ks * ny + ls), i);
        } else if (ks >= 0 && ks < nx && ls >= 0 && ls < ny) {
            v[i] = C::dec(ld1(src + i * n + (long long)ks * ny + ls), i);
        } else {
            v[i] = C::dec(ld1(src + opp(i) * n + (long long)k * ny + l), i);
        }
    }
    if (BC == LBGB_CAVITY_LADD && l == ny - 1) {
        const real lid = real(6) * real(1.0 / 36.0) * u0;
        v[CSE] += lid;  // bounce-back of NW (set above) plus the wall term, every lid node
        v[CSW] -= lid;
    }
    if (BC == LBGB_CAVITY && l == ny - 1) {
        const int T = ny - 1;
        const int kw = (k == 0) ? nx - 1 : k - 1;
        const int ke = (k == nx - 1) ? 0 : k + 1;
        auto g = [&](int ch, int row, int col) { return C::dec(ld1(src + ch * n + (long long)row * ny + col), ch); };
        const real gN = g(CN, k, T), gNW = g(CNW, k, T), gNE = g(CNE, k, T);
        const real rho_lid = gNW + gN + gNE + g(CNW, ke, T - 1) + g(CN, k, T - 1) + g(CNE, kw, T - 1) + g(CW, ke, T) +
                             g(C0, k, T) + g(CE, kw, T);
        const real lid = lid_from_sum<C>(rho_lid, u0);
        if (k != 0) v[CSE] = gNW + lid;
        if (k != nx - 1) v[CSW] = gNE - lid;
    }
}

// R rounds per task: lane j owns cells c0 + 32 r + j, r < R.  The cell
// indices of all R rounds are computed first and all 9 R loads issued before
// the first collision, so each thread keeps 9 R loads in flight (a loop that
// finishes one round before loading the next leaves the kernel waiting on
// load latency).
template <int DT, int BC, int R>
__global__ void __launch_bounds__(256)
k_batch_step_flat(const typename Codec<DT>::raw *__restrict__ src, typename Codec<DT>::raw *__restrict__ dst,
                  long long total_elems, const BatchInstanceDev *__restrict__ inst, int n_inst,
                  const int4 *__restrict__ tasks, long long n_tasks) {
    using C = Codec<DT>;
    using real = typename C::real;
    using raw = typename C::raw;
    const int lane = threadIdx.x & 31;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long t = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < n_tasks; t += nwarps) {
        const int4 tk = tasks[t];
        if (tk.x < 0 || tk.x >= n_inst) continue;
        const BatchInstanceDev in = inst[tk.x];
        const long long n = (long long)in.nx * in.ny;
        if (in.nx <= 0 || in.ny <= 0 || in.offset < 0 || in.offset + 9 * n > total_elems) continue;
        if (BC != LBGB_PERIODIC && (in.nx < 2 || in.ny < 2)) continue;
        if (tk.z < 0) continue;
        const raw *s = src + in.offset;
        raw *d = dst + in.offset;
        // cell c -> (k, l) by one division for the first round, then stepped
        // by 32 cells per round (no 64-bit division per cell)
        long long c = (long long)tk.z + lane;
        int k = (int)(c / in.ny), l = (int)(c - (long long)k * in.ny);
        long long cr[R];
        int kr[R], lr[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            cr[r] = c;
            kr[r] = k;
            lr[r] = l;
            c += 32;
            l += 32;
            while (l >= in.ny) {
                l -= in.ny;
                ++k;
            }
        }
        real v[R][9];
#pragma unroll
        for (int r = 0; r < R; ++r)
            if (cr[r] < n) pull_cell<C, BC>(s, in.nx, in.ny, kr[r], lr[r], (real)in.u0, v[r]);
#pragma unroll
        for (int r = 0; r < R; ++r) {
            if (cr[r] >= n) continue;
            raw out[9];
            collide_encode<DT>(v[r], (real)in.omega, out);
#pragma unroll
            for (int i = 0; i < 9; ++i) d[i * n + cr[r]] = out[i];
        }
    }
}

// Per-instance diagnostics run on a (LBGB_DIAG_CHUNKS, n_inst) grid: block
// (c, b) covers chunk c of instance b's cells and writes one partial; a second
// kernel combines the partials of each instance in chunk order, so results
// do not depend on scheduling.  (One block per instance left the largest
// lattice on a single SM.)
__device__ __forceinline__ void chunk_range(long long n, int c, long long &c0, long long &c1) {
    const long long len = (n + LBGB_DIAG_CHUNKS - 1) / LBGB_DIAG_CHUNKS;
    c0 = (long long)c * len;
    c1 = c0 + len < n ? c0 + len : n;
}

// Amplitude of a sine mode of u_x along y:
// a_b = 2/(nx*ny) * sum_{k,l} u_x(k,l) sin(2 pi l / ny).
template <int DT>
__global__ void __launch_bounds__(256)
k_batch_shear_amplitude(const typename Codec<DT>::raw *__restrict__ f, long long total_elems,
                        const BatchInstanceDev *__restrict__ inst, int n_inst, double *__restrict__ part) {
    using C = Codec<DT>;
    const int b = blockIdx.y, chunk = blockIdx.x;
    if (b >= n_inst) return;
    const BatchInstanceDev in = inst[b];
    const long long n = (long long)in.nx * in.ny;
    double acc = 0.0;
    const bool ok = in.nx > 0 && in.ny > 0 && in.offset >= 0 && in.offset + 9 * n <= total_elems;
    if (ok) {
        const typename C::raw *g = f + in.offset;
        const float two_over_ny = 2.0f / (float)in.ny;
        long long c0, c1;
        chunk_range(n, chunk, c0, c1);
        for (long long c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
            typename C::real v[9];
#pragma unroll
            for (int i = 0; i < 9; ++i) v[i] = C::dec(g[i * n + c], i);
            const typename C::real rho = node_density<DT>(v);
            const double ux = (double)((v[1] - v[3] + v[5] - v[6] - v[7] + v[8]) / rho);
            const int l = (int)(c % in.ny);
            acc += ux * (double)sinpif(two_over_ny * (float)l);
        }
    }
    __shared__ double sm[256];
    sm[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sm[threadIdx.x] += sm[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[(long long)b * LBGB_DIAG_CHUNKS + chunk] = sm[0];
}

__global__ void k_batch_amplitude_finish(const BatchInstanceDev *__restrict__ inst, int n_inst,
                                         const double *__restrict__ part, long long total_elems,
                                         double *__restrict__ out) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n_inst) return;
    const BatchInstanceDev in = inst[b];
    const long long n = (long long)in.nx * in.ny;
    const bool ok = in.nx > 0 && in.ny > 0 && in.offset >= 0 && in.offset + 9 * n <= total_elems;
    double s = 0.0;
    for (int c = 0; c < LBGB_DIAG_CHUNKS; ++c) s += part[(long long)b * LBGB_DIAG_CHUNKS + c];
    out[b] = ok ? s * 2.0 / (double)n : 0.0;
}

// Steady-state monitor: per instance, max over cells of |u - u_prev| (both
// components), then u_prev <- u.  u_prev holds 2 floats per cell, instances
// back to back in cell_base order.
template <int DT>
__global__ void __launch_bounds__(256)
k_batch_velocity_change(const typename Codec<DT>::raw *__restrict__ f, long long total_elems,
                        const BatchInstanceDev *__restrict__ inst, int n_inst, float *__restrict__ u_prev,
                        long long total_cells, double *__restrict__ part) {
    using C = Codec<DT>;
    const int b = blockIdx.y, chunk = blockIdx.x;
    if (b >= n_inst) return;
    const BatchInstanceDev in = inst[b];
    const long long n = (long long)in.nx * in.ny;
    const bool ok = in.nx > 0 && in.ny > 0 && in.offset >= 0 && in.offset + 9 * n <= total_elems &&
                    (long long)in.cell_base + n <= total_cells;
    float m = 0.f;
    if (ok) {
        const typename C::raw *g = f + in.offset;
        float *up = u_prev + 2ll * in.cell_base;
        long long c0, c1;
        chunk_range(n, chunk, c0, c1);
        for (long long c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
            typename C::real v[9];
#pragma unroll
            for (int i = 0; i < 9; ++i) v[i] = C::dec(g[i * n + c], i);
            const typename C::real rho = node_density<DT>(v);
            const float ux = (float)((v[1] - v[3] + v[5] - v[6] - v[7] + v[8]) / rho);
            const float uy = (float)((v[2] - v[4] + v[5] + v[6] - v[7] - v[8]) / rho);
            float d = fmaxf(fabsf(ux - up[2 * c]), fabsf(uy - up[2 * c + 1]));
            if (!(d <= 3.0e38f)) d = INFINITY;  // a NaN (diverged run) must never read as converged
            m = fmaxf(m, d);
            up[2 * c] = ux;
            up[2 * c + 1] = uy;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
    __shared__ float sm[8];
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        float r = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r = fmaxf(r, sm[w]);
        part[(long long)b * LBGB_DIAG_CHUNKS + chunk] = ok ? r : -1.0;
    }
}

__global__ void k_batch_change_finish(int n_inst, const double *__restrict__ part, float *__restrict__ out) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n_inst) return;
    double m = part[(long long)b * LBGB_DIAG_CHUNKS];
    for (int c = 1; c < LBGB_DIAG_CHUNKS; ++c) m = fmax(m, part[(long long)b * LBGB_DIAG_CHUNKS + c]);
    out[b] = (float)m;
}

template <int DT, int BC>
static int launch_batch(const void *src, void *dst, long long total, const void *inst, int n_inst, const void *tasks,
                        long long n_tasks, int rows, int threads, int blocks, int flat, cudaStream_t s) {
    using raw = typename Codec<DT>::raw;
    constexpr int VW = 16 / sizeof(raw);
    if (flat) {
        // rounds per task: 1, 2, 4 or 8 (the task queue steps 32 * rows cells)
        auto go = [&](auto kernel) {
            kernel<<<blocks, threads, 0, s>>>(static_cast<const raw *>(src), static_cast<raw *>(dst), total,
                                              static_cast<const BatchInstanceDev *>(inst), n_inst,
                                              static_cast<const int4 *>(tasks), n_tasks);
        };
        switch (rows) {
        case 1: go(k_batch_step_flat<DT, BC, 1>); break;
        case 2: go(k_batch_step_flat<DT, BC, 2>); break;
        case 4: go(k_batch_step_flat<DT, BC, 4>); break;
        case 8: go(k_batch_step_flat<DT, BC, 8>); break;
        default: set_error("lbgb_batch_step: flat tasks take 1, 2, 4 or 8 rounds (got %d)", rows); return LBGB_EINVAL;
        }
        return check_launch("k_batch_step_flat");
    }
    k_batch_step<DT, BC, VW><<<blocks, threads, 0, s>>>(
        static_cast<const raw *>(src), static_cast<raw *>(dst), total, static_cast<const BatchInstanceDev *>(inst),
        n_inst, static_cast<const int4 *>(tasks), n_tasks, rows);
    return check_launch("k_batch_step");
}

}  // namespace lbgb

extern "C" int lbgb_batch_step(const void *src, void *dst, long long total_elems, const void *instances,
                               int n_instances, const void *tasks, long long n_tasks, int rows_per_task,
                               int boundary, int dtype, int threads, int blocks, int flat, void *stream) {
    using namespace lbgb;
    if (raw_size(dtype) == 0) {
        set_error("lbgb_batch_step: unsupported storage code %d", dtype);
        return LBGB_EDTYPE;
    }
    if (!src || !dst || !instances || !tasks || n_instances <= 0 || n_tasks < 0 || total_elems <= 0) {
        set_error("lbgb_batch_step: null buffer or empty batch");
        return LBGB_EINVAL;
    }
    if (boundary != LBGB_PERIODIC && boundary != LBGB_CAVITY && boundary != LBGB_CAVITY_LADD) {
        set_error("lbgb_batch_step: unknown boundary code %d", boundary);
        return LBGB_EINVAL;
    }
    if (threads < 32 || threads > 256 || threads % 32 || blocks <= 0 || rows_per_task <= 0) {
        set_error("lbgb_batch_step: threads must be a multiple of 32 in [32, 256], blocks and rows > 0");
        return LBGB_EINVAL;
    }
    const size_t bytes = (size_t)total_elems * raw_size(dtype);
    const char *a = static_cast<const char *>(src), *b = static_cast<const char *>(dst);
    if (a < b + bytes && b < a + bytes) {
        set_error("lbgb_batch_step: src and dst overlap");
        return LBGB_EINVAL;
    }
    if (!aligned(src, 16) || !aligned(dst, 16) || !aligned(instances, 8) || !aligned(tasks, 16)) {
        set_error("lbgb_batch_step: buffers must be 16-byte aligned (instance table 8-byte)");
        return LBGB_EINVAL;
    }
    if (n_tasks == 0) return LBGB_OK;
    cudaStream_t s = (cudaStream_t)stream;
#define LBGB_BATCH_CASE(DTV)                                                                                   \
    case DTV:                                                                                                  \
        if (boundary == LBGB_CAVITY)                                                                           \
            return launch_batch<DTV, LBGB_CAVITY>(src, dst, total_elems, instances, n_instances, tasks, n_tasks, \
                                                  rows_per_task, threads, blocks, flat, s);                    \
        if (boundary == LBGB_CAVITY_LADD)                                                                      \
            return launch_batch<DTV, LBGB_CAVITY_LADD>(src, dst, total_elems, instances, n_instances, tasks,   \
                                                       n_tasks, rows_per_task, threads, blocks, flat, s);      \
        return launch_batch<DTV, LBGB_PERIODIC>(src, dst, total_elems, instances, n_instances, tasks, n_tasks,  \
                                                rows_per_task, threads, blocks, flat, s);
    switch (dtype) {
        LBGB_BATCH_CASE(LBGB_F32)
        LBGB_BATCH_CASE(LBGB_F64)
        LBGB_BATCH_CASE(LBGB_F16DEV)
        LBGB_BATCH_CASE(LBGB_BF16DEV)
        LBGB_BATCH_CASE(LBGB_F32DEV)
    }
#undef LBGB_BATCH_CASE
    return LBGB_EDTYPE;
}

extern "C" int lbgb_batch_shear_amplitude(const void *f, long long total_elems, const void *instances,
                                          int n_instances, int dtype, double *out_dev, double *partials,
                                          void *stream) {
    using namespace lbgb;
    if (!f || !instances || !out_dev || !partials || n_instances <= 0 || n_instances > 65535 || total_elems <= 0) {
        set_error("lbgb_batch_shear_amplitude: null buffer, empty batch or more than 65535 instances");
        return LBGB_EINVAL;
    }
    if (!aligned(instances, 8) || !aligned(partials, 8)) {
        set_error("lbgb_batch_shear_amplitude: instance table and partials must be 8-byte aligned");
        return LBGB_EINVAL;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const auto *in = static_cast<const BatchInstanceDev *>(instances);
    const dim3 grid(LBGB_DIAG_CHUNKS, n_instances);
    switch (dtype) {
    case LBGB_F32:
        k_batch_shear_amplitude<LBGB_F32><<<grid, 256, 0, s>>>((const float *)f, total_elems, in, n_instances,
                                                               partials);
        break;
    case LBGB_F64:
        k_batch_shear_amplitude<LBGB_F64><<<grid, 256, 0, s>>>((const double *)f, total_elems, in, n_instances,
                                                               partials);
        break;
    case LBGB_F16DEV:
        k_batch_shear_amplitude<LBGB_F16DEV><<<grid, 256, 0, s>>>((const unsigned short *)f, total_elems, in,
                                                                  n_instances, partials);
        break;
    case LBGB_BF16DEV:
        k_batch_shear_amplitude<LBGB_BF16DEV><<<grid, 256, 0, s>>>((const unsigned short *)f, total_elems, in,
                                                                   n_instances, partials);
        break;
    case LBGB_F32DEV:
        k_batch_shear_amplitude<LBGB_F32DEV><<<grid, 256, 0, s>>>((const float *)f, total_elems, in, n_instances,
                                                                  partials);
        break;
    default: set_error("lbgb_batch_shear_amplitude: unsupported storage code %d", dtype); return LBGB_EDTYPE;
    }
    int rc = check_launch("k_batch_shear_amplitude");
    if (rc) return rc;
    k_batch_amplitude_finish<<<(n_instances + 127) / 128, 128, 0, s>>>(in, n_instances, partials, total_elems,
                                                                       out_dev);
    return check_launch("k_batch_amplitude_finish");
}

extern "C" int lbgb_batch_velocity_change(const void *f, long long total_elems, const void *instances,
                                          int n_instances, int dtype, float *u_prev, long long total_cells,
                                          float *out_dev, double *partials, void *stream) {
    using namespace lbgb;
    if (!f || !instances || !u_prev || !out_dev || !partials || n_instances <= 0 || n_instances > 65535 ||
        total_elems <= 0 || total_cells <= 0) {
        set_error("lbgb_batch_velocity_change: null buffer, empty batch or more than 65535 instances");
        return LBGB_EINVAL;
    }
    if (!aligned(instances, 8) || !aligned(u_prev, 8) || !aligned(partials, 8)) {
        set_error("lbgb_batch_velocity_change: instance table, u_prev and partials must be 8-byte aligned");
        return LBGB_EINVAL;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const auto *in = static_cast<const BatchInstanceDev *>(instances);
    const dim3 grid(LBGB_DIAG_CHUNKS, n_instances);
    switch (dtype) {
    case LBGB_F32:
        k_batch_velocity_change<LBGB_F32><<<grid, 256, 0, s>>>((const float *)f, total_elems, in, n_instances, u_prev,
                                                               total_cells, partials);
        break;
    case LBGB_F64:
        k_batch_velocity_change<LBGB_F64><<<grid, 256, 0, s>>>((const double *)f, total_elems, in, n_instances,
                                                               u_prev, total_cells, partials);
        break;
    case LBGB_F16DEV:
        k_batch_velocity_change<LBGB_F16DEV><<<grid, 256, 0, s>>>((const unsigned short *)f, total_elems, in,
                                                                  n_instances, u_prev, total_cells, partials);
        break;
    case LBGB_BF16DEV:
        k_batch_velocity_change<LBGB_BF16DEV><<<grid, 256, 0, s>>>((const unsigned short *)f, total_elems, in,
                                                                   n_instances, u_prev, total_cells, partials);
        break;
    case LBGB_F32DEV:
        k_batch_velocity_change<LBGB_F32DEV><<<grid, 256, 0, s>>>((const float *)f, total_elems, in, n_instances,
                                                                  u_prev, total_cells, partials);
        break;
    default: set_error("lbgb_batch_velocity_change: unsupported storage code %d", dtype); return LBGB_EDTYPE;
    }
    int rc = check_launch("k_batch_velocity_change");
    if (rc) return rc;
    k_batch_change_finish<<<(n_instances + 127) / 128, 128, 0, s>>>(n_instances, partials, out_dev);
    return check_launch("k_batch_change_finish");
}
