// Two time steps per pass over the lattice (temporal blocking), for 4-byte
// storage (LBGB_F32, LBGB_F32DEV) with periodic or cavity walls: every
// population is read once and written once per two steps, 36 bytes per cell
// update instead of 72.
//
// A block owns `rows` (16-128) consecutive rows x S2_W columns of the output
// and walks its rows in order, two per iteration.  Each f(t) row it needs
// (its own rows and two more on either side, with four columns more on
// either side, both periodic) comes into a ring of S2_NA shared-memory rows
// by 16-byte cp.async, two rows ahead of use.  When rows j, j+1 of f(t) have
// landed, the block computes rows j-1, j of f(t+1) over its columns and one
// more on either side (pull, walls, lid, collision: the single-step kernel's
// arithmetic) into a ring of S2_NB shared-memory rows, stored as the
// storage's own codes, and then rows j-2, j-1 of f(t+2) over its own columns
// from that ring, written to global memory: two independent cells per thread
// and phase.  The rows and columns next to the block's are computed twice,
// by this block and by its neighbour (3 % more collisions at 128 x 256); the
// intermediate step never leaves the SM, so the results equal two single
// steps bit for bit.
#pragma once

namespace lbgb {

constexpr int S2_W = 256;                 // output columns per block
constexpr int S2_THREADS = 288;           // one column of each of two rows per thread (258 for step t+1)
constexpr int S2_NA = 6;                  // f(t) ring: four rows in use, two in flight
constexpr int S2_NB = 4;                  // f(t+1) ring
constexpr int S2_PITCH = S2_W + 8;        // columns Y0-4 .. Y0+W+3 of a channel row
constexpr int S2_VROW = S2_W / 4 + 2;     // 16-byte copies per channel row (main + two halos)
constexpr size_t S2_SMEM = (size_t)(S2_NA + S2_NB) * 9 * S2_PITCH * 4;

// One cell's pull (walls and lid as the single-step kernel), collision and
// encode.  r0, r1, r2: the shared rows of the source step at rows k-1, k, k+1
// (channel-major, S2_PITCH apart); sc: the cell's shared column; k, l: its
// lattice row and column.
template <int DT, int BC>
__device__ __forceinline__ void s2_cell(const typename Codec<DT>::raw *r0, const typename Codec<DT>::raw *r1,
                                        const typename Codec<DT>::raw *r2, int sc, int k, int l, int nx, int ny,
                                        typename Codec<DT>::real omega, typename Codec<DT>::real u0,
                                        typename Codec<DT>::raw (&out)[9]) {
    using C = Codec<DT>;
    using real = typename C::real;
    auto at = [&](int ch, int dr, int dc) {
        const typename C::raw *r = dr < 0 ? r0 : (dr > 0 ? r2 : r1);
        return C::dec(r[ch * S2_PITCH + sc + dc], ch);
    };
    real v[9];
    v[0] = at(C0, 0, 0);
    if (BC == LBGB_PERIODIC || (k != 0 && k != nx - 1)) {
        // every row but the two wall rows (k is the same for the whole block:
        // a uniform branch, one load per value)
#pragma unroll
        for (int ch = 1; ch < 9; ++ch) v[ch] = at(ch, -cx(ch), -cy(ch));
    } else {
#pragma unroll
        for (int ch = 1; ch < 9; ++ch) {
            const bool wall = (cx(ch) > 0 && k == 0) || (cx(ch) < 0 && k == nx - 1);
            v[ch] = wall ? C::dec(r1[opp(ch) * S2_PITCH + sc], ch) : at(ch, -cx(ch), -cy(ch));
        }
    }
    if (BC != LBGB_PERIODIC) {
        if (l == 0) {
            v[CN] = C::dec(r1[CS * S2_PITCH + sc], CN);
            v[CNE] = C::dec(r1[CSW * S2_PITCH + sc], CNE);
            v[CNW] = C::dec(r1[CSE * S2_PITCH + sc], CNW);
        }
        if (l == ny - 1) {
            const real gN = at(CN, 0, 0), gNW = at(CNW, 0, 0), gNE = at(CNE, 0, 0);
            const real rho_lid = gNW + gN + gNE + at(CNW, 1, -1) + at(CN, 0, -1) + at(CNE, -1, -1) + at(CW, 1, 0) +
                                 at(C0, 0, 0) + at(CE, -1, 0);
            const real lid = lid_from_sum<C>(rho_lid, u0);
            v[CS] = gN;
            v[CSE] = (k == 0) ? gNW : gNW + lid;
            v[CSW] = (k == nx - 1) ? gNE : gNE - lid;
        }
    }
    collide_encode<DT>(v, omega, out);
}

template <int DT, int BC>
__global__ void __launch_bounds__(S2_THREADS, 2)
k_step2(const typename Codec<DT>::raw *__restrict__ src, typename Codec<DT>::raw *__restrict__ dst, int nx, int ny,
        int rows, typename Codec<DT>::real omega, typename Codec<DT>::real u0) {
    using raw = typename Codec<DT>::raw;
    static_assert(sizeof(raw) == 4, "four-byte storage");
    extern __shared__ __align__(16) unsigned char s2_smem[];
    raw *A = reinterpret_cast<raw *>(s2_smem);
    raw *B = A + S2_NA * 9 * S2_PITCH;
    const int tid = threadIdx.x;
    const int X0 = blockIdx.x * rows, Y0 = blockIdx.y * S2_W;
    const size_t cs = (size_t)nx * ny;
    // lattice row of input offset o (rows X0-2 .. X0+rows+1, periodic)
    auto row_of = [&](int o) {
        int k = X0 - 2 + o;
        if (k < 0) k += nx;
        if (k >= nx) k -= nx;
        return k;
    };
    auto issue = [&](int o) {
        const raw *base = src + (size_t)row_of(o) * ny;
        raw *slot = A + (o % S2_NA) * 9 * S2_PITCH;
        for (int i = tid; i < 9 * S2_VROW; i += S2_THREADS) {
            const int ch = i / S2_VROW, v = i - ch * S2_VROW;
            int gcol, scol;
            if (v < S2_W / 4) {
                gcol = Y0 + 4 * v;
                scol = 4 + 4 * v;
            } else if (v == S2_W / 4) {
                gcol = Y0 == 0 ? ny - 4 : Y0 - 4;
                scol = 0;
            } else {
                gcol = Y0 + S2_W == ny ? 0 : Y0 + S2_W;
                scol = S2_W + 4;
            }
            cp_async16(slot + ch * S2_PITCH + scol, base + ch * cs + gcol);
        }
    };
    auto arow = [&](int o) { return A + (o % S2_NA) * 9 * S2_PITCH; };
    auto brow = [&](int o) { return B + (o % S2_NB) * 9 * S2_PITCH; };

    // iteration t: inputs 2t, 2t+1 land; step t+1 at offsets 2t-1, 2t (valid
    // 1 .. rows+2), step t+2 at offsets 2t-2, 2t-1 (valid 2 .. rows+1)
    const int n_in = rows + 4, iters = n_in / 2;
    issue(0);
    issue(1);
    cp_async_commit();
    issue(2);
    issue(3);
    cp_async_commit();
    // step t+1 column of this thread (258 of them), step t+2 column (256)
    const bool c1 = tid < S2_W + 2, c2 = tid < S2_W;
    int l1 = Y0 - 1 + tid;
    if (l1 < 0) l1 += ny;
    if (l1 >= ny) l1 -= ny;
    const int sc1 = 3 + tid, l2 = Y0 + tid, sc2 = 4 + tid;
    for (int t = 0; t < iters; ++t) {
        cp_async_wait<1>();  // this thread's copies of inputs 2t, 2t+1 have landed
        __syncthreads();     // ... everyone's; and the previous iteration is done
        if (t >= 1 && c1) {
            const int oa = 2 * t - 1, ob = 2 * t;
            raw outa[9], outb[9];
            s2_cell<DT, BC>(arow(oa - 1), arow(oa), arow(oa + 1), sc1, row_of(oa), l1, nx, ny, omega, u0, outa);
            s2_cell<DT, BC>(arow(ob - 1), arow(ob), arow(ob + 1), sc1, row_of(ob), l1, nx, ny, omega, u0, outb);
            raw *ba = brow(oa), *bb = brow(ob);
#pragma unroll
            for (int ch = 0; ch < 9; ++ch) {
                ba[ch * S2_PITCH + sc1] = outa[ch];
                bb[ch * S2_PITCH + sc1] = outb[ch];
            }
        }
        __syncthreads();
        // the slots of inputs 2t+4, 2t+5 held inputs 2t-2, 2t-1, last read by
        // step t+1 above; they land during step t+2 and the next iteration's wait
        if (2 * t + 4 < n_in) issue(2 * t + 4);
        if (2 * t + 5 < n_in) issue(2 * t + 5);
        cp_async_commit();
        if (t >= 2 && c2) {
            const int oa = 2 * t - 2, ob = 2 * t - 1, ka = row_of(oa), kb = row_of(ob);
            raw outa[9], outb[9];
            s2_cell<DT, BC>(brow(oa - 1), brow(oa), brow(oa + 1), sc2, ka, l2, nx, ny, omega, u0, outa);
            s2_cell<DT, BC>(brow(ob - 1), brow(ob), brow(ob + 1), sc2, kb, l2, nx, ny, omega, u0, outb);
            raw *da = dst + (size_t)ka * ny + l2, *db = dst + (size_t)kb * ny + l2;
#pragma unroll
            for (int ch = 0; ch < 9; ++ch) {
                da[ch * cs] = outa[ch];
                db[ch * cs] = outb[ch];
            }
        }
    }
}

}  // namespace lbgb
