// Two time steps per pass over the lattice (temporal blocking) with periodic
// or cavity walls: every population is read once and written once per two
// steps, 36 bytes per FP32 cell update instead of 72.  Dispatched for FP32
// and f32dev storage; the kernel also takes 2-byte codes (eight per 16-byte
// copy), but the 16-bit single-step kernel is faster.
//
// A block owns `rows` (16-128) consecutive rows x S2_W columns of the output
// and walks its rows in order, two per iteration.  Each f(t) row it needs
// (its own rows and two more on either side, with eight columns more on
// either side, both periodic) comes into a ring of S2_NA shared-memory rows
// by 16-byte cp.async, two rows ahead of use.  When rows j, j+1 of f(t) have
// landed, the block computes rows j-1, j of f(t+1) over its columns and four
// more on either side (pull, walls, lid, collision: the single-step kernel's
// arithmetic) into a ring of S2_NB shared-memory rows, stored as the
// storage's own codes, and then rows j-2, j-1 of f(t+2) over its own columns
// from that ring, written to global memory.  A thread computes four
// consecutive cells of a row (16-byte shared loads plus one edge value for
// the channels that move along y; 16-byte stores).  The rows and columns
// next to the block's are computed twice, by this block and by its
// neighbour (~8 % more collisions at 128 x 128); the intermediate step never
// leaves the SM, so the results equal two single steps bit for bit.
#pragma once

namespace lbgb {

constexpr int S2_W = 128;                 // output columns per block
constexpr int S2_NV = S2_W / 4;           // output four-cell vectors per row (32)
constexpr int S2_NV1 = S2_NV + 2;         // step t+1 vectors per row: one more per side (34)
constexpr int S2_THREADS = 96;            // 2 rows x 34 step t+1 vectors, 2 x 32 step t+2 vectors
constexpr int S2_NA = 6;                  // f(t) ring: four rows in use, two in flight
constexpr int S2_NB = 4;                  // f(t+1) ring
constexpr int S2_PITCH = S2_W + 16;       // columns Y0-8 .. Y0+W+7 of a channel row (elements)

// Per storage size: 16-byte copies per channel row, shared memory per block
// and resident blocks per SM (4-byte codes: 52 KB, four; 2-byte: 26 KB, six
// -- the register limit of 96-thread blocks).
template <class raw>
struct S2Geom {
    static constexpr int VL = 16 / (int)sizeof(raw);  // codes per 16-byte copy
    static constexpr int VROW = S2_PITCH / VL;
    static constexpr size_t SMEM = (size_t)(S2_NA + S2_NB) * 9 * S2_PITCH * sizeof(raw);
    static constexpr int MIN_BLOCKS = sizeof(raw) == 4 ? 4 : 6;
};

// Four consecutive codes of a shared row (16 bytes of 4-byte codes, 8 of
// 2-byte codes; aligned).
__device__ __forceinline__ void s2_ld4(const float *p, float (&o)[4]) {
    const float4 q = *reinterpret_cast<const float4 *>(p);
    o[0] = q.x, o[1] = q.y, o[2] = q.z, o[3] = q.w;
}
__device__ __forceinline__ void s2_ld4(const unsigned short *p, unsigned short (&o)[4]) {
    const uint2 q = *reinterpret_cast<const uint2 *>(p);
    o[0] = (unsigned short)(q.x & 0xffffu), o[1] = (unsigned short)(q.x >> 16);
    o[2] = (unsigned short)(q.y & 0xffffu), o[3] = (unsigned short)(q.y >> 16);
}
__device__ __forceinline__ void s2_st4(float *p, const float (&x)[4]) {
    *reinterpret_cast<float4 *>(p) = make_float4(x[0], x[1], x[2], x[3]);
}
__device__ __forceinline__ void s2_st4(unsigned short *p, const unsigned short (&x)[4]) {
    *reinterpret_cast<uint2 *>(p) = make_uint2((uint32_t)x[0] | ((uint32_t)x[1] << 16),
                                               (uint32_t)x[2] | ((uint32_t)x[3] << 16));
}

// Four consecutive cells (one 16-byte vector) of one row: pull (walls and lid
// as the single-step kernel), collision and encode.  r0, r1, r2: the shared
// rows of the source step at rows k-1, k, k+1 (channel-major, S2_PITCH
// apart); sc: the shared column of the first cell; k, l0: its lattice row
// and column (l0 a multiple of 4).
template <int DT, int BC>
__device__ __forceinline__ void s2_vec(const typename Codec<DT>::raw *r0, const typename Codec<DT>::raw *r1,
                                       const typename Codec<DT>::raw *r2, int sc, int k, int l0, int nx, int ny,
                                       typename Codec<DT>::real omega, typename Codec<DT>::real u0,
                                       typename Codec<DT>::raw (&out)[9][4]) {
    using C = Codec<DT>;
    using raw = typename C::raw;
    using real = typename C::real;
    real v[9][4];
    auto vec = [&](const raw *r, int ch, real (&o)[4], int dch) {
        raw q[4];
        s2_ld4(r + ch * S2_PITCH + sc, q);
#pragma unroll
        for (int j = 0; j < 4; ++j) o[j] = C::dec(q[j], dch);
    };
#pragma unroll
    for (int ch = 0; ch < 9; ++ch) {
        const raw *rp = cx(ch) > 0 ? r0 : (cx(ch) < 0 ? r2 : r1);
        raw q[4];
        s2_ld4(rp + ch * S2_PITCH + sc, q);
        if (cy(ch) > 0) {
            v[ch][0] = C::dec(rp[ch * S2_PITCH + sc - 1], ch);
            v[ch][1] = C::dec(q[0], ch);
            v[ch][2] = C::dec(q[1], ch);
            v[ch][3] = C::dec(q[2], ch);
        } else if (cy(ch) < 0) {
            v[ch][0] = C::dec(q[1], ch);
            v[ch][1] = C::dec(q[2], ch);
            v[ch][2] = C::dec(q[3], ch);
            v[ch][3] = C::dec(rp[ch * S2_PITCH + sc + 4], ch);
        } else {
#pragma unroll
            for (int j = 0; j < 4; ++j) v[ch][j] = C::dec(q[j], ch);
        }
    }
    if (BC != LBGB_PERIODIC) {
        if (k == 0 || k == nx - 1) {
            // side-wall rows: bounce-back from the same node, decoded as ch
#pragma unroll
            for (int ch = 1; ch < 9; ++ch)
                if ((cx(ch) > 0 && k == 0) || (cx(ch) < 0 && k == nx - 1)) vec(r1, opp(ch), v[ch], ch);
        }
        if (l0 == 0) {
            // bottom wall: N, NE, NW bounce back from the same node
            v[CN][0] = C::dec(r1[CS * S2_PITCH + sc], CN);
            v[CNE][0] = C::dec(r1[CSW * S2_PITCH + sc], CNE);
            v[CNW][0] = C::dec(r1[CSE * S2_PITCH + sc], CNW);
        }
        if (l0 + 3 == ny - 1) {
            // lid (the vector's last cell): the single-step kernel's rule and sum order
            const int s3 = sc + 3;
            const real gN = C::dec(r1[CN * S2_PITCH + s3], CN), gNW = C::dec(r1[CNW * S2_PITCH + s3], CNW),
                       gNE = C::dec(r1[CNE * S2_PITCH + s3], CNE);
            const real rho_lid = gNW + gN + gNE + C::dec(r2[CNW * S2_PITCH + s3 - 1], CNW) +
                                 C::dec(r1[CN * S2_PITCH + s3 - 1], CN) + C::dec(r0[CNE * S2_PITCH + s3 - 1], CNE) +
                                 C::dec(r2[CW * S2_PITCH + s3], CW) + C::dec(r1[C0 * S2_PITCH + s3], C0) +
                                 C::dec(r0[CE * S2_PITCH + s3], CE);
            const real lid = lid_from_sum<C>(rho_lid, u0);
            v[CS][3] = gN;
            v[CSE][3] = (k == 0) ? gNW : gNW + lid;
            v[CSW][3] = (k == nx - 1) ? gNE : gNE - lid;
        }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        real f[9];
        raw r[9];
#pragma unroll
        for (int ch = 0; ch < 9; ++ch) f[ch] = v[ch][j];
        collide_encode<DT>(f, omega, r);
#pragma unroll
        for (int ch = 0; ch < 9; ++ch) out[ch][j] = r[ch];
    }
}

template <int DT, int BC>
__global__ void __launch_bounds__(S2_THREADS, S2Geom<typename Codec<DT>::raw>::MIN_BLOCKS)
k_step2(const typename Codec<DT>::raw *__restrict__ src, typename Codec<DT>::raw *__restrict__ dst, int nx, int ny,
        int rows, typename Codec<DT>::real omega, typename Codec<DT>::real u0) {
    using raw = typename Codec<DT>::raw;
    using G = S2Geom<raw>;
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
    // shared column 0 is lattice column Y0 - 8 (periodic)
    auto issue = [&](int o) {
        const raw *base = src + (size_t)row_of(o) * ny;
        raw *slot = A + (o % S2_NA) * 9 * S2_PITCH;
        for (int i = tid; i < 9 * G::VROW; i += S2_THREADS) {
            const int ch = i / G::VROW, v = i - ch * G::VROW;
            int gcol = Y0 - 8 + G::VL * v;
            if (gcol < 0) gcol += ny;
            if (gcol >= ny) gcol -= ny;
            cp_async16(slot + ch * S2_PITCH + G::VL * v, base + ch * cs + gcol);
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
    // step t+1: thread -> (row r1i, vector u1) of 2 x S2_NV1, columns Y0-4 .. Y0+W+3;
    // step t+2: thread -> (row r2i, vector u2) of 2 x S2_NV, columns Y0 .. Y0+W-1
    const bool c1 = tid < 2 * S2_NV1, c2 = tid < 2 * S2_NV;
    const int r1i = tid >= S2_NV1, u1 = tid - r1i * S2_NV1;
    const int r2i = tid >= S2_NV, u2 = tid - r2i * S2_NV;
    int l1 = Y0 - 4 + 4 * u1;
    if (l1 < 0) l1 += ny;
    if (l1 >= ny) l1 -= ny;
    const int sc1 = 4 + 4 * u1, l2 = Y0 + 4 * u2, sc2 = 8 + 4 * u2;
    for (int t = 0; t < iters; ++t) {
        cp_async_wait<1>();  // this thread's copies of inputs 2t, 2t+1 have landed
        __syncthreads();     // ... everyone's; and the previous iteration is done
        if (t >= 1 && c1) {
            const int o = 2 * t - 1 + r1i;
            raw out[9][4];
            s2_vec<DT, BC>(arow(o - 1), arow(o), arow(o + 1), sc1, row_of(o), l1, nx, ny, omega, u0, out);
            raw *b = brow(o);
#pragma unroll
            for (int ch = 0; ch < 9; ++ch) s2_st4(b + ch * S2_PITCH + sc1, out[ch]);
        }
        __syncthreads();
        // the slots of inputs 2t+4, 2t+5 held inputs 2t-2, 2t-1, last read by
        // step t+1 above; they land during step t+2 and the next iteration's wait
        if (2 * t + 4 < n_in) issue(2 * t + 4);
        if (2 * t + 5 < n_in) issue(2 * t + 5);
        cp_async_commit();
        if (t >= 2 && c2) {
            const int o = 2 * t - 2 + r2i, k = row_of(o);
            raw out[9][4];
            s2_vec<DT, BC>(brow(o - 1), brow(o), brow(o + 1), sc2, k, l2, nx, ny, omega, u0, out);
            raw *d = dst + (size_t)k * ny + l2;
#pragma unroll
            for (int ch = 0; ch < 9; ++ch) s2_st4(d + ch * cs, out[ch]);
        }
    }
}

}  // namespace lbgb
