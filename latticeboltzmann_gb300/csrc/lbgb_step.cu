// Pull-scheme streaming (periodic, or cavity walls with a moving lid) with an
// optional fused BGK collision: the hot path of liblbgb.
//
// Work decomposition.  A warp owns one "segment": 32*V consecutive cells of one
// row k (V cells per lane, l fastest).  Every population is read exactly once
// and written exactly once, so the kernel is a pure HBM stream: per cell
// 9 loads and 9 stores of the storage type (72 B/cell in FP32, 36 B in 16-bit).
//
//  * Channels with cx != 0 read the same l range of row k -/+ 1: an aligned
//    vector load.
//  * Channels with cy != 0 need the lane's vector shifted by one cell along l.
//    The lane loads its own aligned vector and takes the missing edge value
//    from the neighbouring lane with a warp shuffle; only lanes at a segment
//    or row edge issue one extra scalar load (the warp-level replacement of
//    the reference's ghost-cell halo exchange, cavity_opt1.py:247-278).
//  * Cavity walls (cavity_opt1.py:177-245): whole wall rows k = 0 and
//    k = nx-1 are warp-uniform, so their bounce-back is a change of the
//    source plane and row, taken by the whole warp.  The bottom and lid nodes
//    (l = 0, l = ny-1) belong to single lanes, which patch their values with
//    a few scalar loads, including the lid density that the reference reads
//    across the periodic seam at the two lid corners.
#include <limits.h>
#include <stdio.h>

#include "lbgb_common.cuh"
#include "lbgb_pipe.cuh"

namespace lbgb {

constexpr unsigned FULL = 0xffffffffu;

template <class C, int V>
__device__ __forceinline__ void load_plane(const typename C::raw *__restrict__ src, size_t cs, int ny,
                                           int ch_src, int ch_dec, int row, int l0, bool act,
                                           typename C::real (&o)[V]) {
    if (act) {
        typename C::raw r[V];
        ldv<typename C::raw, V>(src + (size_t)ch_src * cs + (size_t)row * ny + l0, r);
#pragma unroll
        for (int j = 0; j < V; ++j) o[j] = C::dec(r[j], ch_dec);
    } else {
#pragma unroll
        for (int j = 0; j < V; ++j) o[j] = 0;
    }
}

template <class C>
__device__ __forceinline__ typename C::real load_one(const typename C::raw *__restrict__ src, size_t cs,
                                                     int ny, int ch, int row, int l) {
    return C::dec(ld1(src + (size_t)ch * cs + (size_t)row * ny + l), ch);
}

// o[j] <- value at l0+j-1 (channels moving in +y).
template <class C, int V, int BC>
__device__ __forceinline__ void shift_from_below(typename C::real (&o)[V], const typename C::raw *__restrict__ src,
                                                 size_t cs, int ny, int ch, int row, int l0, int lane,
                                                 bool act) {
    typename C::real prev = __shfl_up_sync(FULL, o[V - 1], 1);
    if (lane == 0 && act) {
        if (l0 > 0)
            prev = load_one<C>(src, cs, ny, ch, row, l0 - 1);
        else if (BC == LBGB_PERIODIC)
            prev = load_one<C>(src, cs, ny, ch, row, ny - 1);
        // cavity, l0 == 0: bottom-wall bounce-back patched by the caller
    }
#pragma unroll
    for (int j = V - 1; j > 0; --j) o[j] = o[j - 1];
    o[0] = prev;
}

// o[j] <- value at l0+j+1 (channels moving in -y).
template <class C, int V, int BC>
__device__ __forceinline__ void shift_from_above(typename C::real (&o)[V], const typename C::raw *__restrict__ src,
                                                 size_t cs, int ny, int ch, int row, int l0, int lane,
                                                 bool act) {
    typename C::real next = __shfl_down_sync(FULL, o[0], 1);
    if (act && (lane == 31 || l0 + V >= ny)) {
        if (l0 + V < ny)
            next = load_one<C>(src, cs, ny, ch, row, l0 + V);
        else if (BC == LBGB_PERIODIC)
            next = load_one<C>(src, cs, ny, ch, row, 0);
        // cavity, last node of the row: lid rule patched by the caller
    }
#pragma unroll
    for (int j = 0; j < V - 1; ++j) o[j] = o[j + 1];
    o[V - 1] = next;
}

// Pulls channel ch of V nodes (k, l0..l0+V-1) into o.  wall = the source row
// lies beyond a cavity side wall: bounce back from the same node instead.
template <class C, int V, int BC, int CH>
__device__ __forceinline__ void pull_channel(typename C::real (&o)[V], const typename C::raw *__restrict__ src,
                                             size_t cs, int ny, int k, int krow, bool wall, int l0, int lane,
                                             bool act) {
    if (wall) {
        load_plane<C, V>(src, cs, ny, opp(CH), CH, k, l0, act, o);
        return;
    }
    load_plane<C, V>(src, cs, ny, CH, CH, krow, l0, act, o);
    if (cy(CH) > 0) shift_from_below<C, V, BC>(o, src, cs, ny, CH, krow, l0, lane, act);
    if (cy(CH) < 0) shift_from_above<C, V, BC>(o, src, cs, ny, CH, krow, l0, lane, act);
}

// Resident blocks per SM the register allocation must allow: the 8-cell
// 16-bit variant needs ~110 registers, the others ~80.
template <int DT, int V>
constexpr int min_blocks() { return (sizeof(typename Codec<DT>::raw) == 2 && V == 8) ? 2 : 3; }

// One warp segment of one row: lane `lane` owns cells (k, l0 .. l0+V-1) of a
// (9, nx, ny) lattice at src/dst.  Shared by the single-lattice kernel and
// the batched multi-lattice kernel.
template <int DT, int BC, bool COLLIDE, int V>
__device__ __forceinline__ void step_segment(const typename Codec<DT>::raw *__restrict__ src,
                                             typename Codec<DT>::raw *__restrict__ dst, int nx, int ny, int k,
                                             int l0, int lane, typename Codec<DT>::real omega,
                                             typename Codec<DT>::real u0,
                                             const unsigned long long *__restrict__ sr_step, uint32_t sr_seed,
                                             uint32_t cell_base) {
    using C = Codec<DT>;
    using real = typename C::real;
    using raw = typename C::raw;
    const size_t cs = (size_t)nx * ny;
    const bool act = l0 < ny;
    int km = k - 1, kp = k + 1;
    bool wl = false, wr = false;
    if (BC == LBGB_PERIODIC) {
        if (km < 0) km += nx;
        if (kp >= nx) kp -= nx;
    } else {
        wl = (k == 0);
        wr = (k == nx - 1);
    }
    real v[9][V];
    pull_channel<C, V, BC, C0>(v[C0], src, cs, ny, k, k, false, l0, lane, act);
    pull_channel<C, V, BC, CE>(v[CE], src, cs, ny, k, km, wl, l0, lane, act);
    pull_channel<C, V, BC, CN>(v[CN], src, cs, ny, k, k, false, l0, lane, act);
    pull_channel<C, V, BC, CW>(v[CW], src, cs, ny, k, kp, wr, l0, lane, act);
    pull_channel<C, V, BC, CS>(v[CS], src, cs, ny, k, k, false, l0, lane, act);
    pull_channel<C, V, BC, CNE>(v[CNE], src, cs, ny, k, km, wl, l0, lane, act);
    pull_channel<C, V, BC, CNW>(v[CNW], src, cs, ny, k, kp, wr, l0, lane, act);
    pull_channel<C, V, BC, CSW>(v[CSW], src, cs, ny, k, kp, wr, l0, lane, act);
    pull_channel<C, V, BC, CSE>(v[CSE], src, cs, ny, k, km, wl, l0, lane, act);

    if (BC != LBGB_PERIODIC && act) {
        if (l0 == 0) {
            // bottom wall: N, NE, NW bounce back from the same node
            v[CN][0] = load_one<C>(src, cs, ny, CS, k, 0);
            v[CNE][0] = load_one<C>(src, cs, ny, CSW, k, 0);
            v[CNW][0] = load_one<C>(src, cs, ny, CSE, k, 0);
        }
        if (l0 + V == ny) {
            if (BC == LBGB_CAVITY_LADD) {
                // standard Ladd wall, density 1: -/+ 6 w u0 at every lid node
                const real lid = real(6) * real(1.0 / 36.0) * u0;
                v[CS][V - 1] = load_one<C>(src, cs, ny, CN, k, ny - 1);
                v[CSE][V - 1] = load_one<C>(src, cs, ny, CNW, k, ny - 1) + lid;
                v[CSW][V - 1] = load_one<C>(src, cs, ny, CNE, k, ny - 1) - lid;
            } else {
                // lid: S bounces back; SE/SW get the Ladd term 6 w rho_lid u0,
                // except at the corner where the side wall wins (plain bounce-back)
                const int T = ny - 1;
                const int kw = (k == 0) ? nx - 1 : k - 1;  // periodic neighbours, as
                const int ke = (k == nx - 1) ? 0 : k + 1;  // the reference's roll reads them
                const real gN = load_one<C>(src, cs, ny, CN, k, T);
                const real gNW = load_one<C>(src, cs, ny, CNW, k, T);
                const real gNE = load_one<C>(src, cs, ny, CNE, k, T);
                const real rho_lid = gNW + gN + gNE + load_one<C>(src, cs, ny, CNW, ke, T - 1) +
                                     load_one<C>(src, cs, ny, CN, k, T - 1) +
                                     load_one<C>(src, cs, ny, CNE, kw, T - 1) +
                                     load_one<C>(src, cs, ny, CW, ke, T) + load_one<C>(src, cs, ny, C0, k, T) +
                                     load_one<C>(src, cs, ny, CE, kw, T);
                const real lid = lid_from_sum<C>(rho_lid, u0);
                v[CS][V - 1] = gN;
                v[CSE][V - 1] = (k == 0) ? gNW : gNW + lid;
                v[CSW][V - 1] = (k == nx - 1) ? gNE : gNE - lid;
            }
        }
    }

    raw out[9][V];
    if (COLLIDE) {
        uint32_t key = 0;
        if constexpr (sizeof(raw) == 2) {
            if (sr_step) key = sr_step_key(sr_seed, *sr_step);
        }
#pragma unroll
        for (int j = 0; j < V; ++j) {
            real f[9];
            raw r[9];
#pragma unroll
            for (int i = 0; i < 9; ++i) f[i] = v[i][j];
            if constexpr (sizeof(raw) == 2) {
                if (sr_step)
                    collide_encode_sr<DT>(f, omega, r, key, cell_base + (uint32_t)((size_t)k * ny + l0 + j));
                else
                    collide_encode<DT>(f, omega, r);
            } else {
                collide_encode<DT>(f, omega, r);
            }
#pragma unroll
            for (int i = 0; i < 9; ++i) out[i][j] = r[i];
        }
    } else {
#pragma unroll
        for (int i = 0; i < 9; ++i)
#pragma unroll
            for (int j = 0; j < V; ++j) out[i][j] = C::enc(v[i][j], i);
    }
    if (act) {
#pragma unroll
        for (int i = 0; i < 9; ++i) stv<raw, V>(dst + (size_t)i * cs + (size_t)k * ny + l0, out[i]);
    }
}

template <int DT, int BC, bool COLLIDE, int V>
__global__ void __launch_bounds__(256, min_blocks<DT, V>())
k_step(const typename Codec<DT>::raw *__restrict__ src, typename Codec<DT>::raw *__restrict__ dst, int nx,
       int ny, int segs, long long tasks, typename Codec<DT>::real omega, typename Codec<DT>::real u0,
       const unsigned long long *__restrict__ sr_step, uint32_t sr_seed, int k_first) {
    const int lane = threadIdx.x & 31;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long t = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < tasks; t += nwarps) {
        const int kr = (int)(t / segs);
        const int k = k_first + kr;
        const int l0 = (int)(t - (long long)kr * segs) * (32 * V) + lane * V;
        step_segment<DT, BC, COLLIDE, V>(src, dst, nx, ny, k, l0, lane, omega, u0, sr_step, sr_seed, 0u);
    }
}

// ---------------------------------------------------------------- launch
static int sm_count() {
    static std::atomic<int> cache[MAX_DEVICES];
    const int dev = current_device();
    int v = cache[dev].load(std::memory_order_acquire);
    if (v) return v;
    std::lock_guard<std::mutex> lock(setup_mutex());
    int n = 0;
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    v = n > 0 ? n : 1;
    cache[dev].store(v, std::memory_order_release);
    return v;
}

struct SR {
    const unsigned long long *step = nullptr;  // device step counter; null: round to nearest
    uint32_t seed = 0;
};

// Rows [first, first + count) of the lattice to update (count < 0: all).
struct Rows {
    int first = 0;
    int count = -1;
    int n(int nx) const { return count < 0 ? nx : count; }
};

template <int DT, int BC, bool COLLIDE, int V>
static int launch_v(const void *src, void *dst, int nx, int ny, double omega, double u0, cudaStream_t s,
                    SR sr = SR(), Rows rows = Rows()) {
    using C = Codec<DT>;
    const int threads = 256;
    const int segs = (ny + 32 * V - 1) / (32 * V);
    const long long tasks = (long long)rows.n(nx) * segs;
    const long long warps_per_block = threads / 32;
    long long blocks = (tasks + warps_per_block - 1) / warps_per_block;
    // at most 16 resident-size waves of blocks; the rest is grid-stride
    const long long cap = (long long)sm_count() * 8 * 16;
    if (blocks > cap) blocks = cap;
    k_step<DT, BC, COLLIDE, V><<<(unsigned)blocks, threads, 0, s>>>(
        static_cast<const typename C::raw *>(src), static_cast<typename C::raw *>(dst), nx, ny, segs, tasks,
        (typename C::real)omega, (typename C::real)u0, sr.step, sr.seed, rows.first);
    return check_launch("k_step");
}

// ---------------------------------------------------------------- tuning
struct Tuning {
    long long kernel = 0;                // 0 auto, 1 register kernel, 2 pipelined kernel
    long long stages = 2;                // pipeline depth (shared-memory stages)
    long long wait_limit = 1ll << 22;    // tries per bounded mbarrier wait
    long long pipe_min_cells = 1 << 16;  // auto: smaller lattices use the register kernel
    long long stall_producer = 0;        // test hook: the producer delivers nothing
    long long two_step = 1;              // auto kernel: two time steps per launch where k_step2 applies
};
static Tuning g_tune;

static int max_dyn_smem() {
    static std::atomic<int> cache[MAX_DEVICES];
    const int dev = current_device();
    int v = cache[dev].load(std::memory_order_acquire);
    if (v) return v;
    std::lock_guard<std::mutex> lock(setup_mutex());
    int n = 0;
    cudaDeviceGetAttribute(&n, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    v = n > 0 ? n : 48 * 1024;
    cache[dev].store(v, std::memory_order_release);
    return v;
}

}  // namespace lbgb
#include "lbgb_step2.cuh"
namespace lbgb {

// Rows per block of the two-step kernel: the largest of 128, 64, 32, 16 that
// divides nx (0: none does).
static int step2_rows(int nx) {
    for (int r = 128; r >= 16; r /= 2)
        if (nx % r == 0) return r;
    return 0;
}

static bool step2_applies(const void *src, const void *dst, int nx, int ny, int boundary, int dtype) {
    // 16-bit codes stay on the single-step kernel: issue-bound already, they
    // measured slower with two steps per launch (8192^2 cavity: 148k against
    // 169k MLUPS FP16, 149k against 171k BF16)
    return g_tune.two_step && g_tune.kernel == 0 && (dtype == LBGB_F32 || dtype == LBGB_F32DEV) &&
           (boundary == LBGB_PERIODIC || boundary == LBGB_CAVITY) && step2_rows(nx) && ny % S2_W == 0 &&
           ny / S2_W <= 65535 && (!src || aligned(src, 16)) && (!dst || aligned(dst, 16));
}

template <int DT, int BC>
static int launch_step2(const void *src, void *dst, int nx, int ny, double omega, double u0, cudaStream_t s) {
    using raw = typename Codec<DT>::raw;
    static std::atomic<bool> attr_set[MAX_DEVICES];
    const int dev = current_device();
    if (!attr_set[dev].load(std::memory_order_acquire)) {
        std::lock_guard<std::mutex> lock(setup_mutex());
        const cudaError_t e =
            cudaFuncSetAttribute(k_step2<DT, BC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S2Geom<raw>::SMEM);
        if (e != cudaSuccess) {
            set_error("k_step2: cannot reserve %zu bytes of shared memory: %s", S2Geom<raw>::SMEM,
                      cudaGetErrorString(e));
            return LBGB_ECUDA;
        }
        attr_set[dev].store(true, std::memory_order_release);
    }
    const int rows = step2_rows(nx);
    k_step2<DT, BC><<<dim3(nx / rows, ny / S2_W), S2_THREADS, S2Geom<raw>::SMEM, s>>>(
        static_cast<const raw *>(src), static_cast<raw *>(dst), nx, ny, rows, (typename Codec<DT>::real)omega,
        (typename Codec<DT>::real)u0);
    return check_launch("k_step2");
}

// Two fused steps src -> dst in one launch; 1 (nothing launched) where the
// two-step kernel does not apply.
static int step2(const void *src, void *dst, int nx, int ny, int boundary, double omega, double u0, int dtype,
                 cudaStream_t s) {
    if (!step2_applies(src, dst, nx, ny, boundary, dtype)) return 1;
    const bool cav = boundary == LBGB_CAVITY;
    switch (dtype) {
    case LBGB_F32:
        return cav ? launch_step2<LBGB_F32, LBGB_CAVITY>(src, dst, nx, ny, omega, u0, s)
                   : launch_step2<LBGB_F32, LBGB_PERIODIC>(src, dst, nx, ny, omega, 0.0, s);
    default:
        return cav ? launch_step2<LBGB_F32DEV, LBGB_CAVITY>(src, dst, nx, ny, omega, u0, s)
                   : launch_step2<LBGB_F32DEV, LBGB_PERIODIC>(src, dst, nx, ny, omega, 0.0, s);
    }
}

template <int DT, int BC, bool COLLIDE>
static int launch_pipe(const void *src, void *dst, int nx, int ny, double omega, double u0, cudaStream_t s,
                       SR sr, Rows rows) {
    using raw = typename Codec<DT>::raw;
    using SH = PipeShape<DT>;
    using G = PipeGeom<raw, SH::NCW, SH::NC>;
    const long long tpr = (ny + G::L - 1) / G::L;
    const long long total = (long long)rows.n(nx) * tpr;
    const int smax = max_dyn_smem();
    const int fit = (int)((smax / SH::CTAS - 256) / (G::STAGE_BYTES + 16));
    int stages = (int)g_tune.stages;
    if (stages > fit) stages = fit;
    if (stages < 2 || total > INT_MAX) return 1;  // caller falls back to the register kernel
    const size_t smem = (size_t)stages * G::STAGE_BYTES + 16 * (size_t)stages;
    const long long slots = (long long)sm_count() * SH::CTAS;
    const int grid = (int)(total < slots ? total : slots);
    const bool srnd = sizeof(raw) == 2 && COLLIDE && sr.step != nullptr;
    // the dynamic shared-memory limit is raised once per kernel variant and device
    static std::atomic<bool> attr_set[MAX_DEVICES][2];
    const int dev = current_device();
    auto go = [&](auto kernel, int variant) -> int {
        if (!attr_set[dev][variant].load(std::memory_order_acquire)) {
            std::lock_guard<std::mutex> lock(setup_mutex());
            cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smax);
            if (e != cudaSuccess) {
                set_error("k_step_pipe: cannot reserve %d bytes of shared memory: %s", smax, cudaGetErrorString(e));
                return LBGB_ECUDA;
            }
            attr_set[dev][variant].store(true, std::memory_order_release);
        }
        kernel<<<grid, (SH::NCW + 1) * 32, smem, s>>>(
            static_cast<const raw *>(src), static_cast<raw *>(dst), nx, ny, (int)tpr, (int)total, stages,
            (typename Codec<DT>::real)omega, (typename Codec<DT>::real)u0, g_tune.wait_limit,
            (int)g_tune.stall_producer, sr.step, sr.seed, rows.first);
        return LBGB_OK;
    };
    const int rc = srnd ? go(k_step_pipe<DT, BC, COLLIDE, SH::NCW, SH::NC, sizeof(raw) == 2 && COLLIDE>, 1)
                        : go(k_step_pipe<DT, BC, COLLIDE, SH::NCW, SH::NC, false>, 0);
    if (rc) return rc;
    return check_launch("k_step_pipe");
}

// Pipelined kernel for lattices whose rows hold whole 16-byte vectors (large
// lattices, or when forced); otherwise the register kernel with the widest
// vector width that divides ny and keeps every row start aligned.
template <int DT, int BC, bool COLLIDE>
static int launch(const void *src, void *dst, int nx, int ny, double omega, double u0, cudaStream_t s,
                  SR sr = SR(), Rows rows = Rows()) {
    constexpr int VW = 16 / sizeof(typename Codec<DT>::raw);
    const bool vec_ok = ny % VW == 0 && aligned(src, 16) && aligned(dst, 16);
    const bool want_pipe = g_tune.kernel == 2 ||
                           (g_tune.kernel == 0 && (long long)nx * ny >= g_tune.pipe_min_cells);
    if (vec_ok && want_pipe) {
        const int rc = launch_pipe<DT, BC, COLLIDE>(src, dst, nx, ny, omega, u0, s, sr, rows);
        if (rc <= 0) return rc;
    }
    if (vec_ok) return launch_v<DT, BC, COLLIDE, VW>(src, dst, nx, ny, omega, u0, s, sr, rows);
    return launch_v<DT, BC, COLLIDE, 1>(src, dst, nx, ny, omega, u0, s, sr, rows);
}

template <int BC, bool COLLIDE>
static int dispatch(const void *src, void *dst, int nx, int ny, int dtype, double omega, double u0,
                    cudaStream_t s, SR sr = SR(), Rows rows = Rows()) {
    switch (dtype) {
    case LBGB_F32: return launch<LBGB_F32, BC, COLLIDE>(src, dst, nx, ny, omega, u0, s, SR(), rows);
    case LBGB_F64: return launch<LBGB_F64, BC, COLLIDE>(src, dst, nx, ny, omega, u0, s, SR(), rows);
    case LBGB_F16DEV: return launch<LBGB_F16DEV, BC, COLLIDE>(src, dst, nx, ny, omega, u0, s, sr, rows);
    case LBGB_BF16DEV: return launch<LBGB_BF16DEV, BC, COLLIDE>(src, dst, nx, ny, omega, u0, s, sr, rows);
    case LBGB_F32DEV: return launch<LBGB_F32DEV, BC, COLLIDE>(src, dst, nx, ny, omega, u0, s, SR(), rows);
    default: set_error("unsupported storage code %d", dtype); return LBGB_EDTYPE;
    }
}

static int check_grid(const void *src, void *dst, int nx, int ny, int dtype, int boundary, const char *what) {
    if (raw_size(dtype) == 0) {
        set_error("%s: unsupported storage code %d", what, dtype);
        return LBGB_EDTYPE;
    }
    if (nx <= 0 || ny <= 0) {
        set_error("%s: grid %d x %d must be positive", what, nx, ny);
        return LBGB_EINVAL;
    }
    if (boundary != LBGB_PERIODIC && (nx < 2 || ny < 2)) {
        set_error("%s: the cavity needs nx >= 2 and ny >= 2 (got %d x %d)", what, nx, ny);
        return LBGB_EINVAL;
    }
    if (boundary != LBGB_CAVITY && boundary != LBGB_PERIODIC && boundary != LBGB_CAVITY_LADD) {
        set_error("%s: unknown boundary code %d", what, boundary);
        return LBGB_EINVAL;
    }
    if (!src || !dst) {
        set_error("%s: null population pointer", what);
        return LBGB_EINVAL;
    }
    const size_t bytes = 9 * (size_t)nx * ny * raw_size(dtype);
    const char *a = static_cast<const char *>(src), *b = static_cast<const char *>(dst);
    if (a < b + bytes && b < a + bytes) {
        set_error("%s: src and dst overlap; streaming is out of place", what);
        return LBGB_EINVAL;
    }
    if (!aligned(src, raw_size(dtype)) || !aligned(dst, raw_size(dtype))) {
        set_error("%s: population pointers must be aligned to the element size", what);
        return LBGB_EINVAL;
    }
    return LBGB_OK;
}

}  // namespace lbgb

using namespace lbgb;

extern "C" int lbgb_stream_periodic(const void *src, void *dst, int nx, int ny, int dtype, void *stream) {
    int rc = check_grid(src, dst, nx, ny, dtype, LBGB_PERIODIC, "lbgb_stream_periodic");
    if (rc) return rc;
    return dispatch<LBGB_PERIODIC, false>(src, dst, nx, ny, dtype, 0.0, 0.0, (cudaStream_t)stream);
}

extern "C" int lbgb_stream_bounce_back(const void *src, void *dst, int nx, int ny, double u0, int dtype,
                                       void *stream) {
    int rc = check_grid(src, dst, nx, ny, dtype, LBGB_CAVITY, "lbgb_stream_bounce_back");
    if (rc) return rc;
    return dispatch<LBGB_CAVITY, false>(src, dst, nx, ny, dtype, 0.0, u0, (cudaStream_t)stream);
}

extern "C" int lbgb_step_fused(const void *src, void *dst, int nx, int ny, int boundary, double omega, double u0,
                               int dtype, void *stream) {
    int rc = check_grid(src, dst, nx, ny, dtype, boundary, "lbgb_step_fused");
    if (rc) return rc;
    if (boundary == LBGB_CAVITY)
        return dispatch<LBGB_CAVITY, true>(src, dst, nx, ny, dtype, omega, u0, (cudaStream_t)stream);
    if (boundary == LBGB_CAVITY_LADD)
        return dispatch<LBGB_CAVITY_LADD, true>(src, dst, nx, ny, dtype, omega, u0, (cudaStream_t)stream);
    return dispatch<LBGB_PERIODIC, true>(src, dst, nx, ny, dtype, omega, 0.0, (cudaStream_t)stream);
}

extern "C" int lbgb_step_fused_rows(const void *src, void *dst, int nx, int ny, int k_begin, int k_end,
                                    int boundary, double omega, double u0, int dtype, void *stream) {
    int rc = check_grid(src, dst, nx, ny, dtype, boundary, "lbgb_step_fused_rows");
    if (rc) return rc;
    if (k_begin < 0 || k_end > nx || k_begin > k_end) {
        set_error("lbgb_step_fused_rows: rows [%d, %d) outside [0, %d)", k_begin, k_end, nx);
        return LBGB_EINVAL;
    }
    if (k_begin == k_end) return LBGB_OK;
    Rows rows;
    rows.first = k_begin;
    rows.count = k_end - k_begin;
    cudaStream_t s = (cudaStream_t)stream;
    if (boundary == LBGB_CAVITY) return dispatch<LBGB_CAVITY, true>(src, dst, nx, ny, dtype, omega, u0, s, SR(), rows);
    if (boundary == LBGB_CAVITY_LADD)
        return dispatch<LBGB_CAVITY_LADD, true>(src, dst, nx, ny, dtype, omega, u0, s, SR(), rows);
    return dispatch<LBGB_PERIODIC, true>(src, dst, nx, ny, dtype, omega, 0.0, s, SR(), rows);
}

extern "C" int lbgb_run_fused(void *a, void *b, int nx, int ny, int boundary, double omega, double u0, int dtype,
                              int nsteps, int *which, void *stream) {
    if (nsteps < 0) {
        set_error("lbgb_run_fused: nsteps must be >= 0");
        return LBGB_EINVAL;
    }
    int rc = check_grid(a, b, nx, ny, dtype, boundary, "lbgb_run_fused");
    if (rc) return rc;
    void *src = a, *dst = b;
    int s = 0;
    // pairs of steps in one launch each where the two-step kernel applies
    for (; s + 1 < nsteps; s += 2) {
        rc = step2(src, dst, nx, ny, boundary, omega, u0, dtype, (cudaStream_t)stream);
        if (rc > 0) break;
        if (rc < 0) return rc;
        void *t = src;
        src = dst;
        dst = t;
    }
    for (; s < nsteps; ++s) {
        rc = lbgb_step_fused(src, dst, nx, ny, boundary, omega, u0, dtype, stream);
        if (rc) return rc;
        void *t = src;
        src = dst;
        dst = t;
    }
    if (which) *which = (src == a) ? 0 : 1;
    return LBGB_OK;
}

extern "C" int lbgb_steps_per_launch(int nx, int ny, int boundary, int dtype) {
    return step2_applies(nullptr, nullptr, nx, ny, boundary, dtype) ? 2 : 1;
}

namespace lbgb {
__global__ void k_bump_step(unsigned long long *ctr) { *ctr += 1; }
}  // namespace lbgb

#include "lbgb_batch.cuh"

extern "C" int lbgb_run_fused_sr(void *a, void *b, int nx, int ny, int boundary, double omega, double u0, int dtype,
                                 int nsteps, unsigned int seed, unsigned long long *step_counter, int *which,
                                 void *stream) {
    if (dtype != LBGB_F16DEV && dtype != LBGB_BF16DEV)
        return lbgb_run_fused(a, b, nx, ny, boundary, omega, u0, dtype, nsteps, which, stream);
    if (nsteps < 0) {
        set_error("lbgb_run_fused_sr: nsteps must be >= 0");
        return LBGB_EINVAL;
    }
    if (!step_counter || !aligned(step_counter, 8)) {
        set_error("lbgb_run_fused_sr: step_counter must be an 8-byte aligned device pointer");
        return LBGB_EINVAL;
    }
    int rc = check_grid(a, b, nx, ny, dtype, boundary, "lbgb_run_fused_sr");
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    SR sr;
    sr.step = step_counter;
    sr.seed = seed;
    void *src = a, *dst = b;
    for (int i = 0; i < nsteps; ++i) {
        rc = boundary == LBGB_CAVITY        ? dispatch<LBGB_CAVITY, true>(src, dst, nx, ny, dtype, omega, u0, s, sr)
             : boundary == LBGB_CAVITY_LADD ? dispatch<LBGB_CAVITY_LADD, true>(src, dst, nx, ny, dtype, omega, u0, s, sr)
                                            : dispatch<LBGB_PERIODIC, true>(src, dst, nx, ny, dtype, omega, 0.0, s, sr);
        if (rc) return rc;
        k_bump_step<<<1, 1, 0, s>>>(step_counter);
        rc = check_launch("k_bump_step");
        if (rc) return rc;
        void *t = src;
        src = dst;
        dst = t;
    }
    if (which) *which = (src == a) ? 0 : 1;
    return LBGB_OK;
}

extern "C" int lbgb_set_tuning(int key, long long value) {
    switch (key) {
    case LBGB_TUNE_KERNEL:
        if (value < 0 || value > 2) break;
        g_tune.kernel = value;
        return LBGB_OK;
    case LBGB_TUNE_STAGES:
        if (value < 2 || value > 64) break;
        g_tune.stages = value;
        return LBGB_OK;
    case LBGB_TUNE_WAIT_LIMIT:
        if (value < 1) break;
        g_tune.wait_limit = value;
        return LBGB_OK;
    case LBGB_TUNE_PIPE_MIN_CELLS:
        if (value < 0) break;
        g_tune.pipe_min_cells = value;
        return LBGB_OK;
    case LBGB_TUNE_TEST_STALL_PRODUCER:
        g_tune.stall_producer = value ? 1 : 0;
        return LBGB_OK;
    case LBGB_TUNE_TWO_STEP:
        g_tune.two_step = value ? 1 : 0;
        return LBGB_OK;
    default:
        set_error("lbgb_set_tuning: unknown key %d", key);
        return LBGB_EINVAL;
    }
    set_error("lbgb_set_tuning: value %lld out of range for key %d", value, key);
    return LBGB_EINVAL;
}

extern "C" long long lbgb_get_tuning(int key) {
    switch (key) {
    case LBGB_TUNE_KERNEL: return g_tune.kernel;
    case LBGB_TUNE_STAGES: return g_tune.stages;
    case LBGB_TUNE_WAIT_LIMIT: return g_tune.wait_limit;
    case LBGB_TUNE_PIPE_MIN_CELLS: return g_tune.pipe_min_cells;
    case LBGB_TUNE_TEST_STALL_PRODUCER: return g_tune.stall_producer;
    case LBGB_TUNE_TWO_STEP: return g_tune.two_step;
    }
    return -1;
}

extern "C" int lbgb_device_status(int reset) {
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        set_error("lbgb_device_status: %s", cudaGetErrorString(e));
        return LBGB_ECUDA;
    }
    int v = 0;
    e = cudaMemcpyFromSymbol(&v, g_pipe_status, sizeof(int));
    if (e == cudaSuccess && reset) {
        const int zero = 0;
        e = cudaMemcpyToSymbol(g_pipe_status, &zero, sizeof(int));
    }
    if (e != cudaSuccess) {
        set_error("lbgb_device_status: %s", cudaGetErrorString(e));
        return LBGB_ECUDA;
    }
    if (v != 0) {
        set_error("a bounded device-side wait gave up (site %d)", v);
        return LBGB_ETIMEOUT;
    }
    return LBGB_OK;
}
