// Two time steps per pass over the lattice (temporal blocking), for 4-byte
// storage (LBGB_F32, LBGB_F32DEV) with periodic or cavity walls: every
// population is read once and written once per two steps, 36 bytes per cell
// update instead of 72.
//
// A block owns S2_R consecutive rows x S2_W columns of the output and walks
// its rows in order.  Each f(t) row it needs (its own rows and two more on
// either side, with four columns more on either side, both periodic) comes
// into a ring of S2_NA shared-memory rows by 16-byte cp.async, three rows
// ahead of use.  When row j of f(t) has landed, the block computes row j-1 of
// f(t+1) over its columns and one more on either side (pull, walls, lid,
// collision: the single-step kernel's arithmetic) into a ring of three
// shared-memory rows, stored as the storage's own codes, and then row j-2 of
// f(t+2) over its own columns from that ring, written to global memory.  The
// rows and columns next to the block's are computed twice, by this block and
// by its neighbour (3 % more collisions at 128 x 256); the intermediate step
// never leaves the SM, so the results equal two single steps bit for bit.
#pragma once

namespace lbgb {

constexpr int S2_W = 256;                 // output columns per block
constexpr int S2_THREADS = 256;           // one output column per thread
constexpr int S2_NA = 6;                  // f(t) ring: three rows in use, three in flight
constexpr int S2_NB = 3;                  // f(t+1) ring
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
#pragma unroll
    for (int ch = 1; ch < 9; ++ch) {
        const bool wall = BC != LBGB_PERIODIC && ((cx(ch) > 0 && k == 0) || (cx(ch) < 0 && k == nx - 1));
        v[ch] = wall ? C::dec(r1[opp(ch) * S2_PITCH + sc], ch) : at(ch, -cx(ch), -cy(ch));
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

    const int n_in = rows + 4;
    issue(0);
    cp_async_commit();
    issue(1);
    cp_async_commit();
    issue(2);
    cp_async_commit();
    for (int j = 0; j < n_in; ++j) {
        // the slot of input j+3 held input j-3, last read by step t+1's row
        // j-2 before the second barrier of the previous iteration
        if (j + 3 < n_in) issue(j + 3);
        cp_async_commit();
        cp_async_wait<3>();  // this thread's copies of input j have landed
        __syncthreads();     // ... everyone's; and the previous iteration is done
        if (j >= 2) {
            // step t+1, row j-1 (offset), columns Y0-1 .. Y0+W (periodic)
            const int o = j - 1, k = row_of(o);
            const raw *r0 = arow(o - 1), *r1 = arow(o), *r2 = arow(o + 1);
            raw *b = brow(o);
            for (int c = tid; c < S2_W + 2; c += S2_THREADS) {
                int l = Y0 - 1 + c;
                if (l < 0) l += ny;
                if (l >= ny) l -= ny;
                const int sc = 3 + c;
                raw out[9];
                s2_cell<DT, BC>(r0, r1, r2, sc, k, l, nx, ny, omega, u0, out);
#pragma unroll
                for (int ch = 0; ch < 9; ++ch) b[ch * S2_PITCH + sc] = out[ch];
            }
        }
        __syncthreads();
        if (j >= 4) {
            // step t+2, row j-2 (offset) = lattice row X0 + j - 4, own columns
            const int o = j - 2, k = row_of(o), l = Y0 + tid, sc = 4 + tid;
            raw out[9];
            s2_cell<DT, BC>(brow(o - 1), brow(o), brow(o + 1), sc, k, l, nx, ny, omega, u0, out);
            raw *d = dst + (size_t)k * ny + l;
#pragma unroll
            for (int ch = 0; ch < 9; ++ch) d[ch * cs] = out[ch];
        }
    }
}

}  // namespace lbgb
