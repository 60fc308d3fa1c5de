// Warp-specialised, shared-memory-pipelined variant of the pull step.
//
// One persistent CTA per SM.  Warp NCW (the producer, one thread) streams the
// source data of each tile into a ring of shared-memory stages with bulk
// asynchronous copies (cp.async.bulk, completion counted on an mbarrier);
// warps 0..NCW-1 (the consumers) gather every population of their cells from
// the stage, release it, collide and store straight to global memory.
//
// A tile is L = NCW*32*NC consecutive cells of one row k (NC = cells per
// consumer thread = one 16-byte vector).  For channel i the producer copies
// row k - cx_i (or, at a cavity side wall, the opposite channel of row k),
// columns [l0 - HALO, l0 + L + HALO) clipped to the row, HALO = one 16-byte
// vector: the one-cell neighbours along l that the cy != 0 channels pull are
// then in shared memory.  Only the cells of the first and last column of a
// row fetch their wrap-around or wall values from global memory.
//
// A stage holds ~37 KB (FP32: 9 channels x 1032 cells); with the default
// two stages ~74 KB per SM are in flight, independent of how long the
// consumers spend in the collision (deeper rings measured slower).
//
// Every mbarrier wait is bounded.  A wait that gives up records a code in a
// device-side status word and makes its warp leave the tile loop; the
// producer then waits (bounded again) for the copies it has issued before it
// exits, so no copy can land in the shared memory of a finished CTA.
#pragma once

#include "lbgb_common.cuh"

namespace lbgb {

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}
// Waits for the phase of the given parity; false if `limit` tries pass first.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, long long limit) {
    for (long long n = 0; n < limit; ++n)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
// Requests the line of p into L1 without waiting for it.
__device__ __forceinline__ void prefetch_l1(const void *p) {
    asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}
// Bulk asynchronous copy global -> shared, completion counted on `bar`.
__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

// device-side status word of the pipelined kernels (0 = fine)
__device__ int g_pipe_status;

constexpr long long PIPE_DRAIN_LIMIT = 1ll << 22;

__device__ __forceinline__ void pipe_report(int code) { atomicCAS(&g_pipe_status, 0, code); }

// Tile geometry: NCW consumer warps, NC cells per consumer thread (one 8- or
// 16-byte packet per channel), a 16-byte halo on each side of the row segment
// (bulk copies start and end on 16-byte boundaries).
template <class RAW, int NCW_, int NC_>
struct PipeGeom {
    static constexpr int NCW = NCW_;
    static constexpr int NC = NC_;
    static constexpr int HALO = 16 / (int)sizeof(RAW);
    static constexpr int L = NCW * 32 * NC;                    // cells per tile
    static constexpr int SLOT = L + 2 * HALO;                  // elements per channel slot
    static constexpr size_t STAGE_BYTES = 9ull * SLOT * sizeof(RAW);
};

// Shapes per storage code: FP32 8 warps x 4 cells, FP64 8 x 2; the 16-bit
// codecs have twice the cells per byte, so 8 warps hold 8 cells each (more
// work per thread between the per-tile fixed costs; 168 registers, no
// spills).  CTAS: resident CTAs per SM (the launch bound and the persistent
// grid).  Measured at 8192^2 (FP16, FP16 stochastic, BF16 MLUPS): 8 x 8 with
// one CTA 163.8k / 154.7k / 168.4k; 8 x 4 with two CTAs (96 registers)
// 153.4k / 136.8k / 151.8k; 16 x 4 with one CTA 158.4k / 146.6k / 160.6k.
template <int DT> struct PipeShape { static constexpr int NCW = 8, NC = 4, CTAS = 1; };
template <> struct PipeShape<LBGB_F64> { static constexpr int NCW = 8, NC = 2, CTAS = 1; };
template <> struct PipeShape<LBGB_F16DEV> { static constexpr int NCW = 8, NC = 8, CTAS = 1; };
template <> struct PipeShape<LBGB_BF16DEV> { static constexpr int NCW = 8, NC = 8, CTAS = 1; };

template <int DT, int BC, bool COLLIDE, int NCW_, int NC_, bool SRND>
__global__ void __launch_bounds__((NCW_ + 1) * 32, PipeShape<DT>::CTAS)
k_step_pipe(const typename Codec<DT>::raw *__restrict__ src, typename Codec<DT>::raw *__restrict__ dst, int nx,
            int ny, int tiles_per_row, int total_tiles, int stages, typename Codec<DT>::real omega,
            typename Codec<DT>::real u0, long long wait_limit, int stall_producer,
            const unsigned long long *__restrict__ sr_step, uint32_t sr_seed, int k_first) {
    using C = Codec<DT>;
    using raw = typename C::raw;
    using real = typename C::real;
    using G = PipeGeom<raw, NCW_, NC_>;
    using P = Packet<DT, NC_>;
    constexpr int NC = G::NC, HALO = G::HALO, L = G::L, SLOT = G::SLOT, NCW = G::NCW;
    // FP16 collisions run in the stored units (deviations times 2^14): no
    // scaling per value on decode or encode, bit for bit the same results
    constexpr bool UNITS = DT == LBGB_F16DEV && COLLIDE;
    constexpr int LOG2K = UNITS ? 14 : 0;
    auto decv = [&](raw x, int ch) -> real {
        if constexpr (UNITS)
            return P::dec1_units(x);
        else
            return C::dec(x, ch);
    };

    extern __shared__ __align__(128) unsigned char smem[];
    raw *slots = reinterpret_cast<raw *>(smem);
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + (size_t)stages * G::STAGE_BYTES);
    uint64_t *empty = full + stages;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const size_t cs = (size_t)nx * ny;

    if (threadIdx.x == 0) {
        for (int s = 0; s < stages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], NCW * 32);
        }
        fence_mbar_init();
    }
    __syncthreads();

    if (warp == NCW) {
        // ------------------------------------------------------------ producer
        if (lane != 0) return;
        // test hook for the failure path: a producer that never delivers lets
        // the consumers' bounded waits run out (nothing is in flight)
        if (stall_producer) return;
        int issued = 0;
        for (int tile = blockIdx.x; tile < total_tiles; tile += gridDim.x) {
            const int s = issued % stages;
            const uint32_t ph = (uint32_t)(issued / stages) & 1u;
            if (!mbar_wait(&empty[s], ph ^ 1u, wait_limit)) {
                pipe_report(1);
                break;
            }
            const int k = k_first + tile / tiles_per_row;
            const int l0 = (tile - (k - k_first) * tiles_per_row) * L;
            const int c0 = max(l0 - HALO, 0), c1 = min(l0 + L + HALO, ny);
            const uint32_t bytes = (uint32_t)(c1 - c0) * (uint32_t)sizeof(raw);
            mbar_arrive_expect_tx(&full[s], 9u * bytes);
            raw *stage = slots + (size_t)s * 9 * SLOT;
#pragma unroll
            for (int i = 0; i < 9; ++i) {
                int ch = i, row = k - cx(i);
                if (BC == LBGB_PERIODIC) {
                    row = row < 0 ? row + nx : (row >= nx ? row - nx : row);
                } else if (row < 0 || row >= nx) {
                    ch = opp(i);
                    row = k;
                }
                bulk_copy_g2s(stage + i * SLOT + (c0 - (l0 - HALO)), src + (size_t)ch * cs + (size_t)row * ny + c0,
                              bytes, &full[s]);
            }
            ++issued;
        }
        // drain: the copies of the last stages issued must land before exit
        for (int j = max(0, issued - stages); j < issued; ++j)
            mbar_wait(&full[j % stages], (uint32_t)(j / stages) & 1u, PIPE_DRAIN_LIMIT);
        return;
    }

    // ---------------------------------------------------------------- consumers
    const int t = threadIdx.x;  // 0 .. NCW*32-1
    // tile -> (row, tile within the row), advanced without a division per tile
    const int dq = gridDim.x / tiles_per_row, dr = gridDim.x - dq * tiles_per_row;
    int kr = blockIdx.x / tiles_per_row, lt = blockIdx.x - kr * tiles_per_row;
    // The threads at a row's first and last column read a few values from
    // global memory after the stage wait (wrap-around, walls, the lid
    // density).  Their addresses are prefetched into L1 one tile ahead, so
    // that those warps do not wait a DRAM round trip while holding a stage.
    // (16-bit storage: not done -- those kernels are issue-bound, and the
    // per-tile instructions cost more than the stalls they save: -4 %)
    auto prefetch_edges = [&](int tl, int krow, int ltile) {
        if constexpr (sizeof(raw) == 2) return;
        if (tl >= total_tiles) return;
        const int kk = k_first + krow;
        const int cc = ltile * L + t * NC;
        const bool first = cc == 0, last = cc + NC == ny;
        if (!first && !last) return;
        auto pf = [&](int ch, int row, int l) { prefetch_l1(src + (size_t)ch * cs + (size_t)row * ny + l); };
        if (BC == LBGB_PERIODIC) {
            const int km = kk == 0 ? nx - 1 : kk - 1, kp = kk == nx - 1 ? 0 : kk + 1;
            if (first) {
                pf(CN, kk, ny - 1);
                pf(CNE, km, ny - 1);
                pf(CNW, kp, ny - 1);
            }
            if (last) {
                pf(CS, kk, 0);
                pf(CSW, kp, 0);
                pf(CSE, km, 0);
            }
        } else {
            if (first) {
                pf(CS, kk, 0);
                pf(CSW, kk, 0);
                pf(CSE, kk, 0);
            }
            if (last) {
                const int T = ny - 1;
                pf(CN, kk, T);
                pf(CNW, kk, T);
                pf(CNE, kk, T);
                if (BC == LBGB_CAVITY) {
                    const int kw = kk == 0 ? nx - 1 : kk - 1, ke = kk == nx - 1 ? 0 : kk + 1;
                    pf(CNW, ke, T - 1);
                    pf(CN, kk, T - 1);
                    pf(CNE, kw, T - 1);
                    pf(CW, ke, T);
                    pf(C0, kk, T);
                    pf(CE, kw, T);
                }
            }
        }
    };
    prefetch_edges(blockIdx.x, kr, lt);
    int it = 0;
    for (int tile = blockIdx.x; tile < total_tiles; tile += gridDim.x, ++it) {
        const int k = k_first + kr;
        const int l0 = lt * L;
        lt += dr;
        kr += dq;
        if (lt >= tiles_per_row) {
            lt -= tiles_per_row;
            ++kr;
        }
        prefetch_edges(tile + gridDim.x, kr, lt);
        const int s = it % stages;
        const uint32_t ph = (uint32_t)(it / stages) & 1u;
        if (!mbar_wait(&full[s], ph, wait_limit)) {
            pipe_report(2);
            break;
        }
        const int c = l0 + t * NC;  // first cell of this thread
        const bool act = c < ny;
        const raw *stage = slots + (size_t)s * 9 * SLOT;
        const bool wl = (BC != LBGB_PERIODIC) && k == 0;
        const bool wr = (BC != LBGB_PERIODIC) && k == nx - 1;
        real v[9][NC];
        if (act) {
#pragma unroll
            for (int i = 0; i < 9; ++i) {
                const raw *sl = stage + i * SLOT + HALO + t * NC;
                if constexpr (UNITS)
                    P::dec_units(*reinterpret_cast<const typename P::vec *>(sl), v[i]);
                else
                    P::dec(*reinterpret_cast<const typename P::vec *>(sl), wgt<real>(i), v[i]);
                const bool wall = (cx(i) > 0 && wl) || (cx(i) < 0 && wr);
                if (wall || cy(i) == 0) continue;
                int row = k - cx(i);
                if (BC == LBGB_PERIODIC) row = row < 0 ? row + nx : (row >= nx ? row - nx : row);
                if (cy(i) > 0) {
                    real prev = 0;
                    if (c > 0)
                        prev = decv(sl[-1], i);
                    else if (BC == LBGB_PERIODIC)
                        prev = decv(ld1(src + (size_t)i * cs + (size_t)row * ny + (ny - 1)), i);
#pragma unroll
                    for (int j = NC - 1; j > 0; --j) v[i][j] = v[i][j - 1];
                    v[i][0] = prev;
                } else {
                    real next = 0;
                    if (c + NC < ny)
                        next = decv(sl[NC], i);
                    else if (BC == LBGB_PERIODIC)
                        next = decv(ld1(src + (size_t)i * cs + (size_t)row * ny), i);
#pragma unroll
                    for (int j = 0; j < NC - 1; ++j) v[i][j] = v[i][j + 1];
                    v[i][NC - 1] = next;
                }
            }
        }
        mbar_arrive(&empty[s]);  // this thread is done with the stage
        if (!act) continue;

        if (BC != LBGB_PERIODIC) {
            auto g = [&](int ch, int row, int l) { return decv(ld1(src + (size_t)ch * cs + (size_t)row * ny + l), ch); };
            if (c == 0) {
                v[CN][0] = g(CS, k, 0);
                v[CNE][0] = g(CSW, k, 0);
                v[CNW][0] = g(CSE, k, 0);
            }
            if (c + NC == ny) {
                const int T = ny - 1;
                if (BC == LBGB_CAVITY_LADD) {
                    const real lid = real(6) * real(1.0 / 36.0) * u0 * real(1u << LOG2K);
                    v[CS][NC - 1] = g(CN, k, T);
                    v[CSE][NC - 1] = g(CNW, k, T) + lid;
                    v[CSW][NC - 1] = g(CNE, k, T) - lid;
                } else {
                    const int kw = (k == 0) ? nx - 1 : k - 1;
                    const int ke = (k == nx - 1) ? 0 : k + 1;
                    const real gN = g(CN, k, T), gNW = g(CNW, k, T), gNE = g(CNE, k, T);
                    const real rho_lid = gNW + gN + gNE + g(CNW, ke, T - 1) + g(CN, k, T - 1) + g(CNE, kw, T - 1) +
                                         g(CW, ke, T) + g(C0, k, T) + g(CE, kw, T);
                    real lid;
                    if constexpr (UNITS)
                        lid = lid_term_dev<LOG2K>(rho_lid, u0);
                    else
                        lid = lid_from_sum<C>(rho_lid, u0);
                    v[CS][NC - 1] = gN;
                    v[CSE][NC - 1] = (k == 0) ? gNW : gNW + lid;
                    v[CSW][NC - 1] = (k == nx - 1) ? gNE : gNE - lid;
                }
            }
        }

        raw *out_row = dst + (size_t)k * ny + c;
        if constexpr (COLLIDE && sizeof(raw) == 2) {
            // 16-bit deviations: collide in FP32 in deviation form, pack two
            // values per conversion.  Both codecs write the rest population
            // last, from the stored values, so that each node keeps its mass
            // (see collide_encode); with stochastic rounding (sr_step set)
            // every value is rounded stochastically (see collide_encode_sr).
            constexpr bool sr = SRND;
            if constexpr (DT == LBGB_F16DEV && !SRND) {
                // FP16, round to nearest: the operations of collide_encode<F16DEV>
                // (deviation-form collision, scaled deviations), two values per
                // conversion
                real hs[9][NC];
#pragma unroll
                for (int j = 0; j < NC; ++j) {
                    real h[9];
#pragma unroll
                    for (int i = 0; i < 9; ++i) h[i] = v[i][j];
                    hs[0][j] = collide_dev<false, LOG2K>(h, omega);
#pragma unroll
                    for (int i = 1; i < 9; ++i) hs[i][j] = h[i];
                }
                typename P::vec pk[9];
#pragma unroll
                for (int i = 1; i < 9; ++i) {
                    pk[i] = P::enc_scaled(hs[i]);
                    uint32_t wd[NC / 2];
                    memcpy(wd, &pk[i], sizeof(wd));
#pragma unroll
                    for (int q = 0; q < NC / 2; ++q)
                        fma16x2<false>(wd[q], F16_MINUS_ONE_BITS, hs[0][2 * q], hs[0][2 * q + 1], hs[0][2 * q],
                                       hs[0][2 * q + 1]);
                }
                pk[0] = P::enc_scaled(hs[0]);
#pragma unroll
                for (int i = 0; i < 9; ++i)
                    st_cs(reinterpret_cast<typename P::vec *>(out_row + (size_t)i * cs), pk[i]);
                continue;
            }
            // the rest population keeps the node's mass through the stored
            // values (both roundings, see collide_encode)
            constexpr bool keep_mass = true;
            real hpost[9][NC];
            real dm[NC];
#pragma unroll
            for (int j = 0; j < NC; ++j) {
                real h[9];
#pragma unroll
                for (int i = 0; i < 9; ++i) h[i] = v[i][j];
                dm[j] = collide_dev<!keep_mass, LOG2K>(h, omega);
#pragma unroll
                for (int i = 0; i < 9; ++i) hpost[i][j] = (sr && !UNITS) ? sr_dev<DT>(h[i]) : h[i];
            }
            uint32_t base[NC / 2];
            if constexpr (sr) {
                const uint32_t key = sr_step_key(sr_seed, *sr_step);
                const uint32_t cell0 = (uint32_t)((size_t)k * ny + c);
#pragma unroll
                for (int q = 0; q < NC / 2; ++q) base[q] = sr_pair_base(key, cell0 + 2 * q);
            }
            // each moving channel is stored as soon as it is encoded (fewer
            // live registers); the rest population last, after the mass fix
#pragma unroll
            for (int i = 1; i < 9; ++i) {
                typename P::vec pk;
                if constexpr (sr)
                    pk = enc_h_sr<DT, NC>(hpost[i], base, i);
                else
                    pk = P::enc_h(hpost[i]);
                if constexpr (keep_mass) {
                    uint32_t wd[NC / 2];
                    memcpy(wd, &pk, sizeof(wd));
#pragma unroll
                    for (int q = 0; q < NC / 2; ++q) {
                        if constexpr (UNITS)
                            fma16x2<false>(wd[q], F16_MINUS_ONE_BITS, dm[2 * q], dm[2 * q + 1], dm[2 * q],
                                           dm[2 * q + 1]);
                        else
                            sub_stored2<DT>(dm[2 * q], dm[2 * q + 1], wd[q]);
                    }
                }
                st_cs(reinterpret_cast<typename P::vec *>(out_row + (size_t)i * cs), pk);
            }
            if constexpr (keep_mass) {
#pragma unroll
                for (int j = 0; j < NC; ++j) hpost[0][j] = (sr && !UNITS) ? sr_rest<DT>(dm[j]) : dm[j];
            }
            typename P::vec pk0;
            if constexpr (sr)
                pk0 = enc_h_sr<DT, NC>(hpost[0], base, 0);
            else
                pk0 = P::enc_h(hpost[0]);
            st_cs(reinterpret_cast<typename P::vec *>(out_row), pk0);
        } else {
            raw out[9][NC];
            if (COLLIDE) {
#pragma unroll
                for (int j = 0; j < NC; ++j) {
                    real f[9];
                    raw r[9];
#pragma unroll
                    for (int i = 0; i < 9; ++i) f[i] = v[i][j];
                    collide_encode<DT>(f, omega, r);
#pragma unroll
                    for (int i = 0; i < 9; ++i) out[i][j] = r[i];
                }
            } else {
#pragma unroll
                for (int i = 0; i < 9; ++i)
#pragma unroll
                    for (int j = 0; j < NC; ++j) out[i][j] = C::enc(v[i][j], i);
            }
#pragma unroll
            for (int i = 0; i < 9; ++i) stv<raw, NC>(out_row + (size_t)i * cs, out[i]);
        }
    }
}

}  // namespace lbgb
