// In-place streaming for the drop-in operators (PyLB.Streaming.stream and the
// cavity scripts' stream_and_bounce_back act on their argument in place).
//
// A pull stream reads every node's eight neighbours, so it cannot overwrite
// its source in one pass over independent blocks: a block would read values
// that a neighbouring block has already replaced.  Here the lattice is cut
// into tiles of IP_TX rows x 512 bytes of a row; one block owns one tile, reads
// the whole tile (all nine channels) into shared memory, waits for its own
// threads, and writes the streamed tile back over the same cells.  The only
// values a tile needs from outside itself are the rows and columns next to
// it, and only the three channels that cross each edge; a first kernel saves
// exactly those edge values of every tile into a small workspace before any
// tile is overwritten, and the second kernel takes its halo from there.
//
// Bytes per cell: 72 (FP32: 36 read, 36 written) plus the edge records (the
// pipelined kernel streams runs of tiles along y in order and needs column
// records only at run ends); the stream-into-scratch-and-copy-back it
// replaces moved 144.
// Results equal the out-of-place kernels' bit for bit (same decode, same lid
// arithmetic, same encode).
#include <limits.h>

#include "lbgb_common.cuh"

namespace lbgb {
namespace {

constexpr int IP_TX = 16;         // tile rows (x)
constexpr int IP_THREADS = 256;

template <class raw>
struct IpGeom {
    static constexpr int VW = 16 / (int)sizeof(raw);   // elements per 16-byte vector
    static constexpr int TY = 512 / (int)sizeof(raw);  // tile columns (y): 512 bytes of a row
    static constexpr int PITCH = TY + 2 * VW;          // shared row: halo column, interior at VW, halo column
    static constexpr int ROWS = IP_TX + 2;             // halo row, IP_TX interior rows, halo row
    static constexpr size_t SMEM = 9ull * ROWS * PITCH * sizeof(raw);
    static constexpr int VPR = TY / VW;                // vectors per full tile row (32)
};

// The channels that a neighbouring tile pulls across each edge of a tile:
// side 0 first row (pulled from k+1: cx < 0), side 1 last row (cx > 0),
// side 2 first column (pulled from l+1: cy < 0), side 3 last column (cy > 0).
__host__ __device__ constexpr int edge_ch(int side, int j) {
    return side == 0 ? (j == 0 ? CW : j == 1 ? CNW : CSW)
         : side == 1 ? (j == 0 ? CE : j == 1 ? CNE : CSE)
         : side == 2 ? (j == 0 ? CS : j == 1 ? CSW : CSE)
                     : (j == 0 ? CN : j == 1 ? CNE : CNW);
}

// Tiles are streamed in runs of `run` consecutive tiles along y, one run by
// one block in order (the generic kernel: runs of one tile).  Workspace: row
// records [ntx][2][3][ny] (first / last row of each x tile), then, from a
// 16-byte boundary, column records [nseg][2][3][nx] (first / last column of
// each run; with runs of one tile, of each tile).
struct IpLayout {
    long long ntx, nty, nseg, col_off, total;  // counts and offsets in elements
    int run;
};

template <class raw>
__host__ __device__ inline IpLayout ip_layout(int nx, int ny, int run = 1) {
    using G = IpGeom<raw>;
    IpLayout L;
    L.run = run;
    L.ntx = (nx + IP_TX - 1) / IP_TX;
    L.nty = (ny + G::TY - 1) / G::TY;
    L.nseg = (L.nty + run - 1) / run;
    const long long rows = 6 * L.ntx * (long long)ny;
    L.col_off = (rows + G::VW - 1) / G::VW * G::VW;
    L.total = L.col_off + 6 * L.nseg * (long long)nx;
    return L;
}

// One block per edge record: copies channel edge_ch(side, j) of one row or
// column of f into the workspace.
template <class raw>
__global__ void __launch_bounds__(IP_THREADS) k_ip_save(const raw *f, raw *__restrict__ ws, int nx, int ny,
                                                        int run) {
    using G = IpGeom<raw>;
    const IpLayout L = ip_layout<raw>(nx, ny, run);
    const size_t cs = (size_t)nx * ny;
    const long long rec = blockIdx.x;
    if (rec < 6 * L.ntx) {
        const int t = (int)(rec / 6), side = (int)(rec / 3 % 2), j = (int)(rec % 3);
        const int row = side == 0 ? t * IP_TX : min((t + 1) * IP_TX, nx) - 1;
        const raw *src = f + (size_t)edge_ch(side, j) * cs + (size_t)row * ny;
        raw *dst = ws + rec * ny;
        for (int l = threadIdx.x; l < ny; l += IP_THREADS) dst[l] = src[l];
    } else {
        const long long r2 = rec - 6 * L.ntx;
        const int u = (int)(r2 / 6), side = (int)(r2 / 3 % 2), j = (int)(r2 % 3);
        const int col = side == 0 ? u * run * G::TY : min((u + 1) * run * G::TY, ny) - 1;
        const raw *src = f + (size_t)edge_ch(2 + side, j) * cs + col;
        raw *dst = ws + L.col_off + r2 * nx;
        for (int k = threadIdx.x; k < nx; k += IP_THREADS) dst[k] = src[(size_t)k * ny];
    }
}

// A tile's rows [a, a + txn) and columns [c, c + tyn).
struct IpTile {
    int tx, ty, a, c, txn, tyn;
};

template <class raw>
__device__ __forceinline__ IpTile ip_tile(long long t, const IpLayout &L, int nx, int ny) {
    using G = IpGeom<raw>;
    IpTile T;
    T.tx = (int)(t / L.nty);
    T.ty = (int)(t - (long long)T.tx * L.nty);
    T.a = T.tx * IP_TX;
    T.c = T.ty * G::TY;
    T.txn = min(IP_TX, nx - T.a);
    T.tyn = min(G::TY, ny - T.c);
    return T;
}

// Element offset of (channel, shared row rr, shared column cc) in one stage:
// rr = r + 1 for tile row r (0 and txn + 1 are the halo rows), cc = VW + col
// (VW - 1 and VW + tyn are the halo columns).
template <class raw>
__device__ __forceinline__ int ip_S(int ch, int rr, int cc) {
    using G = IpGeom<raw>;
    return (ch * G::ROWS + rr) * G::PITCH + cc;
}

// Halo value i of tile T, 0 <= i < 6 (tyn + 2) + 6 txn: rows a - 1 and a + txn
// over columns c - 1 .. c + tyn (periodic in both directions), then columns
// c - 1 and c + tyn over the tile's rows.  Sets its shared-memory offset and
// workspace index; false past the end.
template <class raw>
__device__ __forceinline__ bool ip_halo_item(int i, const IpTile &T, const IpLayout &L, int nx, int ny, int &soff,
                                             long long &widx) {
    using G = IpGeom<raw>;
    const int w = T.tyn + 2, nrow = 6 * w;
    if (i < nrow) {
        const int hi = i / (3 * w), rem = i - hi * 3 * w, j = rem / w, col = rem - j * w - 1;
        int l = T.c + col;
        if (l < 0) l += ny;
        if (l >= ny) l -= ny;
        const int tlo = (T.tx == 0 ? (int)L.ntx : T.tx) - 1, thi = (T.tx + 1 == L.ntx) ? 0 : T.tx + 1;
        const long long rec = hi ? ((long long)thi * 2 + 0) * 3 + j : ((long long)tlo * 2 + 1) * 3 + j;
        soff = ip_S<raw>(edge_ch(hi ? 0 : 1, j), hi ? T.txn + 1 : 0, G::VW + col);
        widx = rec * ny + l;
        return true;
    }
    i -= nrow;
    if (i < 6 * T.txn) {
        const int hi = i / (3 * T.txn), rem = i - hi * 3 * T.txn, j = rem / T.txn, r = rem - j * T.txn;
        // runs of one tile: the tile's own column records
        const int ulo = (T.ty == 0 ? (int)L.nseg : T.ty) - 1, uhi = (T.ty + 1 == L.nseg) ? 0 : T.ty + 1;
        const long long rec = hi ? ((long long)uhi * 2 + 0) * 3 + j : ((long long)ulo * 2 + 1) * 3 + j;
        soff = ip_S<raw>(edge_ch(hi ? 2 : 3, j), r + 1, hi ? G::VW + T.tyn : G::VW - 1);
        widx = L.col_off + rec * nx + T.a + r;
        return true;
    }
    return false;
}

// Every value of tile T from the stage s (interior and halo filled), pulled,
// reflected at the cavity walls and lid, written back over the tile in f.
// NT threads, a multiple of the tile width: thread tid owns column tid % TY.
template <int DT, int BC, int NT>
__device__ __forceinline__ void ip_stream_tile(const typename Codec<DT>::raw *s, typename Codec<DT>::raw *f,
                                               const IpTile &T, int nx, int ny, typename Codec<DT>::real u0,
                                               int tid) {
    using C = Codec<DT>;
    using raw = typename C::raw;
    using real = typename C::real;
    using G = IpGeom<raw>;
    static_assert(NT % G::TY == 0, "whole rows per pass");
    constexpr int RPP = NT / G::TY;  // rows per pass
    const size_t cs = (size_t)nx * ny;
    const int col = tid % G::TY;
    if (col >= T.tyn) return;
    const int l = T.c + col, cc = G::VW + col;
    for (int r = tid / G::TY; r < T.txn; r += RPP) {
        const int k = T.a + r, rr = r + 1;
        auto at = [&](int ch, int dr, int dc) { return C::dec(s[ip_S<raw>(ch, rr + dr, cc + dc)], ch); };
        real v[9];
        v[0] = at(C0, 0, 0);
#pragma unroll
        for (int ch = 1; ch < 9; ++ch) {
            const bool wall = BC != LBGB_PERIODIC && ((cx(ch) > 0 && k == 0) || (cx(ch) < 0 && k == nx - 1));
            // side-wall bounce-back from the same node, decoded as channel ch
            v[ch] = wall ? C::dec(s[ip_S<raw>(opp(ch), rr, cc)], ch) : at(ch, -cx(ch), -cy(ch));
        }
        if (BC != LBGB_PERIODIC) {
            if (l == 0) {
                // bottom wall: N, NE, NW bounce back from the same node
                v[CN] = C::dec(s[ip_S<raw>(CS, rr, cc)], CN);
                v[CNE] = C::dec(s[ip_S<raw>(CSW, rr, cc)], CNE);
                v[CNW] = C::dec(s[ip_S<raw>(CSE, rr, cc)], CNW);
            }
            if (l == ny - 1) {
                // lid: S bounces back, SE/SW get the Ladd term with the lid
                // density read across the periodic seam, side walls win at
                // the corners (the out-of-place kernel's sum order)
                const real gN = at(CN, 0, 0), gNW = at(CNW, 0, 0), gNE = at(CNE, 0, 0);
                const real rho_lid = gNW + gN + gNE + at(CNW, 1, -1) + at(CN, 0, -1) + at(CNE, -1, -1) +
                                     at(CW, 1, 0) + at(C0, 0, 0) + at(CE, -1, 0);
                const real lid = lid_from_sum<C>(rho_lid, u0);
                v[CS] = gN;
                v[CSE] = (k == 0) ? gNW : gNW + lid;
                v[CSW] = (k == nx - 1) ? gNE : gNE - lid;
            }
        }
        raw *dst = f + (size_t)k * ny + l;
#pragma unroll
        for (int ch = 0; ch < 9; ++ch) dst[ch * cs] = C::enc(v[ch], ch);
    }
}

// Generic form, any alignment: one block per tile; the tile and its saved
// halo into shared memory, then the streamed tile back over itself.
template <int DT, int BC>
__global__ void __launch_bounds__(IP_THREADS, 2)
k_ip_stream(typename Codec<DT>::raw *f, const typename Codec<DT>::raw *__restrict__ ws, int nx, int ny,
            typename Codec<DT>::real u0) {
    using raw = typename Codec<DT>::raw;
    using G = IpGeom<raw>;
    extern __shared__ __align__(16) unsigned char ip_smem[];
    raw *s = reinterpret_cast<raw *>(ip_smem);
    const IpLayout L = ip_layout<raw>(nx, ny);
    const IpTile T = ip_tile<raw>(blockIdx.x, L, nx, ny);
    const size_t cs = (size_t)nx * ny;
    const int tid = threadIdx.x;
    const int per_ch = T.txn * T.tyn, n = 9 * per_ch;
    for (int i = tid; i < n; i += IP_THREADS) {
        const int ch = i / per_ch, rem = i - ch * per_ch, r = rem / T.tyn, col = rem - r * T.tyn;
        s[ip_S<raw>(ch, r + 1, G::VW + col)] = f[ch * cs + (size_t)(T.a + r) * ny + T.c + col];
    }
    const int nh = 6 * (T.tyn + 2) + 6 * T.txn;
    for (int i = tid; i < nh; i += IP_THREADS) {
        int soff;
        long long widx;
        if (ip_halo_item<raw>(i, T, L, nx, ny, soff, widx)) s[soff] = ws[widx];
    }
    __syncthreads();
    ip_stream_tile<DT, BC, IP_THREADS>(s, f, T, nx, ny, u0, tid);
}

// Pipelined form for rows of whole 16-byte vectors (16-byte aligned f, ny a
// multiple of the vector width): one persistent block per SM with two
// stages, streaming runs of IP_RUN consecutive tiles along y, each run in
// order.  While a tile is streamed out of one stage, the next tile's interior
// is on its way into the other (16-byte cp.async, one group per tile) and its
// halo values into registers, so the SM's loads and stores overlap instead of
// alternating.  Within a run a tile's left halo column is the previous tile's
// old last column, copied from that tile's stage, and its right halo column is
// the next tile's first column, read from f before that tile is written (an
// L2 hit: the next tile is loaded one iteration later); only the run ends
// need column records, and a block touches no tile of another run.
constexpr int IPP_THREADS = 512;
constexpr int IP_RUN = 4;

// Halo value i of tile T at position (first, last) of run sg: rows a - 1 and
// a + txn over columns c - 1 .. c + tyn from the row records, then the left
// column (the run's record at its first tile; otherwise carried: nullptr) and
// the right column (the next run's record at its last tile; otherwise the
// next tile's first column in f).  Sets the shared-memory offset and returns
// the address to read; nullptr past the end or for a carried value.
template <class raw, bool FULL>
__device__ __forceinline__ const raw *ip_run_halo(int i, const IpTile &T, int sg, bool first, bool last,
                                                  const IpLayout &L, int nx, int ny, const raw *f, const raw *ws,
                                                  size_t cs, int &soff) {
    using G = IpGeom<raw>;
    const int txn = FULL ? IP_TX : T.txn, tyn = FULL ? G::TY : T.tyn;
    const int w = tyn + 2, nrow = 6 * w;
    if (i < nrow) {
        const int hi = i / (3 * w), rem = i % (3 * w), j = rem / w, col = rem % w - 1;
        int l = T.c + col;
        if (l < 0) l += ny;
        if (l >= ny) l -= ny;
        const int tlo = (T.tx == 0 ? (int)L.ntx : T.tx) - 1, thi = (T.tx + 1 == L.ntx) ? 0 : T.tx + 1;
        const long long rec = hi ? ((long long)thi * 2 + 0) * 3 + j : ((long long)tlo * 2 + 1) * 3 + j;
        soff = ip_S<raw>(edge_ch(hi ? 0 : 1, j), hi ? txn + 1 : 0, G::VW + col);
        return ws + rec * ny + l;
    }
    i -= nrow;
    if (i >= 6 * txn) return nullptr;
    const int hi = i / (3 * txn), rem = i % (3 * txn), j = rem / txn, r = rem % txn;
    const int ch = edge_ch(hi ? 2 : 3, j);
    soff = ip_S<raw>(ch, r + 1, hi ? G::VW + tyn : G::VW - 1);
    if (hi) {
        if (!last) return f + ch * cs + (size_t)(T.a + r) * ny + T.c + tyn;
        const int uhi = (sg + 1 == L.nseg) ? 0 : sg + 1;
        return ws + L.col_off + (((long long)uhi * 2 + 0) * 3 + j) * nx + T.a + r;
    }
    if (!first) return nullptr;
    const int ulo = (sg == 0 ? (int)L.nseg : sg) - 1;
    return ws + L.col_off + (((long long)ulo * 2 + 1) * 3 + j) * nx + T.a + r;
}

template <int DT, int BC>
__global__ void __launch_bounds__(IPP_THREADS, 1)
k_ip_stream_pipe(typename Codec<DT>::raw *f, const typename Codec<DT>::raw *__restrict__ ws, int nx, int ny,
                 typename Codec<DT>::real u0) {
    using raw = typename Codec<DT>::raw;
    using G = IpGeom<raw>;
    constexpr int STAGE = 9 * G::ROWS * G::PITCH;                                    // elements per stage
    constexpr int QMAX = 9 * IP_TX * G::VPR / IPP_THREADS;                           // vectors per thread
    constexpr int HMAX = (6 * (G::TY + 2) + 6 * IP_TX + IPP_THREADS - 1) / IPP_THREADS;  // halo values per thread
    static_assert(9 * IP_TX * G::VPR % IPP_THREADS == 0, "full tiles split evenly over the threads");
    extern __shared__ __align__(16) unsigned char ip_smem[];
    raw *sm = reinterpret_cast<raw *>(ip_smem);
    const IpLayout L = ip_layout<raw>(nx, ny, IP_RUN);
    const size_t cs = (size_t)nx * ny;
    const int tid = threadIdx.x;
    const long long nunits = L.ntx * L.nseg;

    // position: run `unit` (x tile, run along y), tile p of it
    struct Pos {
        long long unit;
        int p;
    };
    auto run_len = [&](long long u) {
        const long long left = L.nty - (u % L.nseg) * L.run;
        return (int)(left < L.run ? left : L.run);
    };
    auto next = [&](Pos q) -> Pos {
        if (q.p + 1 < run_len(q.unit)) return Pos{q.unit, q.p + 1};
        return Pos{q.unit + gridDim.x, 0};
    };
    auto tile = [&](Pos q) -> IpTile {
        IpTile T;
        T.tx = (int)(q.unit / L.nseg);
        T.ty = (int)(q.unit - (long long)T.tx * L.nseg) * L.run + q.p;
        T.a = T.tx * IP_TX;
        T.c = T.ty * G::TY;
        T.txn = min(IP_TX, nx - T.a);
        T.tyn = min(G::TY, ny - T.c);
        return T;
    };

    auto issue = [&](const IpTile &T, raw *stage) {
        const raw *src = f + (size_t)T.a * ny + T.c;
        if (T.txn == IP_TX && T.tyn == G::TY) {
            // full tile: the index split by constants (shifts)
#pragma unroll
            for (int q = 0; q < QMAX; ++q) {
                const int i = tid + q * IPP_THREADS;
                const int ch = i / (IP_TX * G::VPR), rem = i % (IP_TX * G::VPR), r = rem / G::VPR,
                          v = rem % G::VPR;
                cp_async16(stage + ip_S<raw>(ch, r + 1, G::VW + v * G::VW),
                           src + ch * cs + (size_t)r * ny + v * G::VW);
            }
            return;
        }
        const int vpr = T.tyn / G::VW, per_ch = T.txn * vpr, nvec = 9 * per_ch;
#pragma unroll
        for (int q = 0; q < QMAX; ++q) {
            const int i = tid + q * IPP_THREADS;
            if (i < nvec) {
                const int ch = i / per_ch, rem = i - ch * per_ch, r = rem / vpr, v = rem - r * vpr;
                cp_async16(stage + ip_S<raw>(ch, r + 1, G::VW + v * G::VW),
                           src + ch * cs + (size_t)r * ny + v * G::VW);
            }
        }
    };
    raw hv[HMAX];
    int hs[HMAX];
    auto fetch_halo = [&](Pos q) {
        const IpTile T = tile(q);
        const int sg = (int)(q.unit % L.nseg);
        const bool first = q.p == 0, last = q.p + 1 == run_len(q.unit);
        const bool full = T.txn == IP_TX && T.tyn == G::TY;
#pragma unroll
        for (int k = 0; k < HMAX; ++k) {
            int soff = -1;
            const raw *src = full ? ip_run_halo<raw, true>(tid + k * IPP_THREADS, T, sg, first, last, L, nx, ny, f,
                                                           ws, cs, soff)
                                  : ip_run_halo<raw, false>(tid + k * IPP_THREADS, T, sg, first, last, L, nx, ny, f,
                                                            ws, cs, soff);
            hs[k] = src ? soff : -1;
            if (src) hv[k] = *src;
        }
    };

    Pos cur{blockIdx.x, 0};
    if (cur.unit >= nunits) return;
    int st = 0;
    issue(tile(cur), sm);
    cp_async_commit();
    fetch_halo(cur);
    while (cur.unit < nunits) {
        const Pos nx_pos = next(cur);
        const bool more = nx_pos.unit < nunits;
        const IpTile T = tile(cur);
        raw *stg = sm + st * STAGE, *stn = sm + (st ^ 1) * STAGE;
        // the other stage was last read by the previous tile, which every
        // thread finished before the barrier that ended the last iteration
        if (more) issue(tile(nx_pos), stn);
        cp_async_commit();  // one group per iteration, empty at the end
#pragma unroll
        for (int k = 0; k < HMAX; ++k)
            if (hs[k] >= 0) stg[hs[k]] = hv[k];
        if (more) fetch_halo(nx_pos);
        cp_async_wait<1>();  // this thread's copies of the current tile have landed
        __syncthreads();       // ... and everyone's, with the halo
        if (more && nx_pos.p > 0) {
            // the next tile of this run takes this tile's old last column as
            // its left halo (channels that cross that edge: N, NE, NW)
            for (int i = tid; i < 3 * T.txn; i += IPP_THREADS) {
                const int j = i / T.txn, r = i - j * T.txn, ch = edge_ch(3, j);
                stn[ip_S<raw>(ch, r + 1, G::VW - 1)] = stg[ip_S<raw>(ch, r + 1, G::VW + T.tyn - 1)];
            }
        }
        ip_stream_tile<DT, BC, IPP_THREADS>(stg, f, T, nx, ny, u0, tid);
        __syncthreads();
        st ^= 1;
        cur = nx_pos;
    }
}

int ip_sm_count() {
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

template <int DT>
int launch_ip(void *f, int nx, int ny, int boundary, double u0, void *ws, size_t ws_bytes, cudaStream_t s,
              const char *what) {
    using raw = typename Codec<DT>::raw;
    using G = IpGeom<raw>;
    const IpLayout L = ip_layout<raw>(nx, ny);
    const size_t need = (size_t)L.total * sizeof(raw);
    if (!ws || ws_bytes < need) {
        set_error("%s: workspace of %zu bytes given, %zu needed (lbgb_stream_inplace_workspace_bytes)", what,
                  ws_bytes, need);
        return LBGB_EINVAL;
    }
    if (!aligned(ws, 16)) {
        set_error("%s: the workspace must be 16-byte aligned", what);
        return LBGB_EINVAL;
    }
    const long long tiles = L.ntx * L.nty, recs = 6 * (L.ntx + L.nty);
    if (tiles > INT_MAX || recs > INT_MAX) {
        set_error("%s: lattice %d x %d has too many tiles", what, nx, ny);
        return LBGB_EINVAL;
    }
    const bool vec = (ny % G::VW == 0) && aligned(f, 16);
    const int run = vec ? IP_RUN : 1;
    const IpLayout LR = ip_layout<raw>(nx, ny, run);
    raw *fp = static_cast<raw *>(f);
    k_ip_save<raw><<<(unsigned)(6 * (LR.ntx + LR.nseg)), IP_THREADS, 0, s>>>(fp, static_cast<raw *>(ws), nx, ny, run);
    int rc = check_launch("k_ip_save");
    if (rc) return rc;
    // variants: periodic / cavity x generic / pipelined
    static std::atomic<bool> attr_set[MAX_DEVICES][4];
    const int dev = current_device();
    const int variant = (boundary == LBGB_PERIODIC ? 0 : 1) + (vec ? 2 : 0);
    const size_t smem = vec ? 2 * G::SMEM : G::SMEM;
    auto go = [&](auto kernel, unsigned grid, int threads, const char *name) -> int {
        if (!attr_set[dev][variant].load(std::memory_order_acquire)) {
            std::lock_guard<std::mutex> lock(setup_mutex());
            cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) {
                set_error("%s: cannot reserve %zu bytes of shared memory: %s", name, smem, cudaGetErrorString(e));
                return LBGB_ECUDA;
            }
            attr_set[dev][variant].store(true, std::memory_order_release);
        }
        kernel<<<grid, threads, smem, s>>>(fp, static_cast<const raw *>(ws), nx, ny, (typename Codec<DT>::real)u0);
        return check_launch(name);
    };
    if (vec) {
        const long long units = LR.ntx * LR.nseg;
        const unsigned grid = (unsigned)(units < ip_sm_count() ? units : ip_sm_count());
        return boundary == LBGB_PERIODIC
                   ? go(k_ip_stream_pipe<DT, LBGB_PERIODIC>, grid, IPP_THREADS, "k_ip_stream_pipe")
                   : go(k_ip_stream_pipe<DT, LBGB_CAVITY>, grid, IPP_THREADS, "k_ip_stream_pipe");
    }
    return boundary == LBGB_PERIODIC ? go(k_ip_stream<DT, LBGB_PERIODIC>, (unsigned)tiles, IP_THREADS, "k_ip_stream")
                                     : go(k_ip_stream<DT, LBGB_CAVITY>, (unsigned)tiles, IP_THREADS, "k_ip_stream");
}

int ip_check(void *f, int nx, int ny, int dtype, int boundary, const char *what) {
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
    if (!f) {
        set_error("%s: null population pointer", what);
        return LBGB_EINVAL;
    }
    if (!aligned(f, raw_size(dtype))) {
        set_error("%s: population pointer must be aligned to the element size", what);
        return LBGB_EINVAL;
    }
    return LBGB_OK;
}

int ip_dispatch(void *f, int nx, int ny, int dtype, int boundary, double u0, void *ws, size_t ws_bytes,
                void *stream, const char *what) {
    int rc = ip_check(f, nx, ny, dtype, boundary, what);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    switch (dtype) {
    case LBGB_F32: return launch_ip<LBGB_F32>(f, nx, ny, boundary, u0, ws, ws_bytes, s, what);
    case LBGB_F64: return launch_ip<LBGB_F64>(f, nx, ny, boundary, u0, ws, ws_bytes, s, what);
    case LBGB_F16DEV: return launch_ip<LBGB_F16DEV>(f, nx, ny, boundary, u0, ws, ws_bytes, s, what);
    case LBGB_BF16DEV: return launch_ip<LBGB_BF16DEV>(f, nx, ny, boundary, u0, ws, ws_bytes, s, what);
    case LBGB_F32DEV: return launch_ip<LBGB_F32DEV>(f, nx, ny, boundary, u0, ws, ws_bytes, s, what);
    default: set_error("%s: unsupported storage code %d", what, dtype); return LBGB_EDTYPE;
    }
}

}  // namespace
}  // namespace lbgb

using namespace lbgb;

extern "C" size_t lbgb_stream_inplace_workspace_bytes(int nx, int ny, int dtype) {
    if (nx <= 0 || ny <= 0) return 0;
    switch (raw_size(dtype)) {
    case 2: return (size_t)ip_layout<unsigned short>(nx, ny).total * 2;
    case 4: return (size_t)ip_layout<float>(nx, ny).total * 4;
    case 8: return (size_t)ip_layout<double>(nx, ny).total * 8;
    default: return 0;
    }
}

extern "C" int lbgb_stream_periodic_inplace(void *f, int nx, int ny, int dtype, void *work, size_t work_bytes,
                                            void *stream) {
    return ip_dispatch(f, nx, ny, dtype, LBGB_PERIODIC, 0.0, work, work_bytes, stream,
                       "lbgb_stream_periodic_inplace");
}

extern "C" int lbgb_stream_bounce_back_inplace(void *f, int nx, int ny, double u0, int dtype, void *work,
                                               size_t work_bytes, void *stream) {
    return ip_dispatch(f, nx, ny, dtype, LBGB_CAVITY, u0, work, work_bytes, stream,
                       "lbgb_stream_bounce_back_inplace");
}
