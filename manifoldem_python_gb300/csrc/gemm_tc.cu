// Split-BF16 tcgen05 form of the all-pairs CTF distance (reference :391-397).
//
//   D_ij = a_i + a_j + E_ij,  E_ij = u'_i.v'_j + v'_i.u'_j - r'_i.r'_j - s'_i.s'_j
//
// Each feature x is stored as x_hi = bf16(x), x_lo = bf16(x - x_hi); E is accumulated as
// A_hi.B_hi + A_hi.B_lo + A_lo.B_hi (the lo.lo term, ~2^-16 relative, is dropped except in the
// chunks the schedule marks, the low-frequency ring-sum chunks of U', V') on the 5th-gen
// tensor cores: tcgen05.mma kind::f16 (BF16 in, FP32 accumulate in TMEM), operands staged in
// shared memory by TMA (128-byte swizzle).  B reads the same feature matrix as A with its first
// two column blocks swapped: each 64-wide K chunk takes its A and B columns from the plan's
// chunk schedule (TMA coordinates); the r', s' chunks use the instruction descriptor's
// negate-B bit, so one accumulator holds E.
//
// One CTA per upper-triangle 128 x 128 tile (pd, I, J); 10 warps:
//   warps 0-7  epilogue: warp w reads TMEM lanes 32*(w%4).. and columns 64*(w/4)..;
//   warp 8     TMA producer (3-stage ring of 64 KB stages: A_hi, A_lo, B_hi, B_lo, K = 64);
//   warp 9     TMEM allocator and MMA issuer.
// The K loop is cut into groups of `group_chunks` 64-wide chunks; each group accumulates into
// one of two TMEM buffers and the epilogue warps add the finished group into FP32 register sums
// (compensated), so the tensor core's FP32 accumulation only ever spans one group.
// Every mbarrier wait is bounded: on expiry the CTA sets the status word's timeout bit, stops
// issuing, waits (bounded) for its own TMA copies and MMAs, frees its TMEM and returns.
#include <algorithm>
#include <type_traits>

#include "tcgen05.cuh"

namespace mem {
namespace {

using namespace tc;

constexpr int TC_M = 128, TC_BK = 64;
constexpr int TC_EPI_WARPS = 8;
constexpr int TC_THREADS = (TC_EPI_WARPS + 2) * 32;
constexpr int TC_OPB = TC_M * TC_BK * 2;          // one 128-row operand box: 16 KB
constexpr int TC_MAX_STAGES = 3;

// Tile shape 128 x BN (BN = 128 or 256 columns of D): a stage holds A_hi, A_lo (128 rows each)
// and B_hi, B_lo (BN rows each, BN / 128 boxes) of one 64-wide K chunk; three 64 KB stages
// at BN = 128, two 96 KB stages at BN = 256
template <int BN>
struct TcShape {
    static constexpr int B_BOXES = BN / 128;
    static constexpr int STAGE_BYTES = (2 + 2 * B_BOXES) * TC_OPB;
    static constexpr int STAGES = BN == 256 ? 2 : 3;
    static constexpr size_t SMEM = (size_t)STAGES * STAGE_BYTES + 1024 + 256;
    // epilogue warps: 4 lane quadrants x BN / 64 column blocks of 64, so that every epilogue
    // thread keeps 64 running sums (BN = 256 with 8 warps would keep 128 and spill)
    static constexpr int EPI_WARPS = BN / 16;
    static constexpr int THREADS = (EPI_WARPS + 2) * 32;
    static_assert(STAGES <= TC_MAX_STAGES, "stage ring");
};

// instruction descriptor, kind::f16: D f32 (bits 4-5 = 1), A bf16 (7-9 = 1), B bf16 (10-12 = 1),
// K-major A and B (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at bits 24-28, negate B bit 14
template <int BN>
__host__ __device__ constexpr uint32_t idesc_f16() {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
           ((uint32_t)(TC_M >> 4) << 24);
}

constexpr int TC_MAX_BUFS = 4;

struct TcShared {
    uint64_t full[TC_MAX_STAGES];
    uint64_t empty[TC_MAX_STAGES];
    uint64_t acc_full[TC_MAX_BUFS];
    uint64_t acc_empty[TC_MAX_BUFS];
    uint64_t mma_done;
    uint32_t tmem_base;
    int abort_flag;
};

// The contraction over the tiles [tile_begin, tile_begin + tile_count) of the plan's tile list:
// CTA b takes tiles tile_begin + b + k gridDim.x (a persistent CTA when the grid is smaller
// than the tile count; one tile per CTA when it is as large).  The producer, the MMA issuer and
// the epilogue each walk the CTA's tiles in the same order; the stage ring and the NBUF TMEM
// accumulators (NBUF x 128 columns) continue from one tile to the next, so a tile's first
// groups are loaded and multiplied while the epilogue still adds and stores the previous tile.
template <bool KAHAN, bool LOLO, int NBUF, int BN>
__global__ void __launch_bounds__(TcShape<BN>::THREADS, 1) gemm_tc_kernel(
        const __grid_constant__ CUtensorMap map_hi, const __grid_constant__ CUtensorMap map_lo,
        const double* __restrict__ pair_norm, const uint32_t* __restrict__ scale_bits,
        const Tile* __restrict__ tiles, const PdDev* __restrict__ pds, double* __restrict__ D,
        uint32_t* __restrict__ status, const int4* __restrict__ chunks, int nchunks,
        int group_chunks, long long wait_limit, int withhold, int tile_begin, int tile_count) {
    static_assert(NBUF == 2 || NBUF == 4, "two or four TMEM accumulators");
    static_assert(BN == 128 || BN == 256, "tile widths");
    static_assert(NBUF * BN <= 512, "TMEM holds 512 columns");
    using S = TcShape<BN>;
    constexpr int TC_STAGES = S::STAGES, TC_STAGE_BYTES = S::STAGE_BYTES;
    constexpr uint32_t IDESC = idesc_f16<BN>(), IDESC_NEG = IDESC | (1u << 14);
    constexpr int EPI = S::EPI_WARPS;              // epilogue warps (warps 0 .. EPI - 1)
    constexpr int EC = 64;                         // epilogue columns per thread
    constexpr uint32_t TMEM_COLS = NBUF * BN;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    TcShared* sh = (TcShared*)(smem + TC_STAGES * TC_STAGE_BYTES);
    volatile int* abort_flag = &sh->abort_flag;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int my_tiles = (int)blockIdx.x < tile_count
                             ? (tile_count - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x
                             : 0;
    auto tile_of = [&](int lt) { return tiles[tile_begin + (int)blockIdx.x + lt * (int)gridDim.x]; };
    const int gsize = (group_chunks > 0 && group_chunks < nchunks) ? group_chunks : nchunks;
    const int ngroups = (nchunks + gsize - 1) / gsize;

    if (threadIdx.x == 0) {
        for (int s = 0; s < TC_STAGES; ++s) {
            mbar_init(&sh->full[s], 1);
            mbar_init(&sh->empty[s], 1);
        }
        for (int b = 0; b < NBUF; ++b) {
            mbar_init(&sh->acc_full[b], 1);
            mbar_init(&sh->acc_empty[b], EPI);
        }
        mbar_init(&sh->mma_done, 1);
        sh->abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == EPI + 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(&sh->tmem_base)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = sh->tmem_base;

    if (warp == EPI) {
        // ---------------------------------------------------------------- TMA producer
        if (lane == 0) {
            asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&map_hi) : "memory");
            asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&map_lo) : "memory");
            long long gc = 0, withheld = -1;     // chunks issued by this CTA (all its tiles)
            bool stop = false;
            for (int lt = 0; lt < my_tiles && !stop; ++lt) {
                const Tile t = tile_of(lt);
                const PdDev pd = pds[t.pd];
                const int rowA = (int)(pd.row_off + (int64_t)t.I * TC_M);
                const int rowB = (int)(pd.row_off + (int64_t)t.J * BN);
                for (int c = 0; c < nchunks; ++c, ++gc) {
                    const int st = (int)(gc % TC_STAGES);
                    const uint32_t ph = (uint32_t)(gc / TC_STAGES) & 1u;
                    if (gc >= TC_STAGES &&
                        !mbar_wait(&sh->empty[st], ph ^ 1u, abort_flag, status, wait_limit)) {
                        stop = true;
                        break;
                    }
                    // a withheld chunk (test of the timeout path; first tile only) is never
                    // loaded, so the MMA issuer's wait for it can only end by its limit
                    if (lt == 0 && c == withhold) {
                        withheld = gc;
                        continue;
                    }
                    // the chunk schedule interleaves the feature blocks so that the dominant
                    // low-frequency columns of every block are accumulated last
                    const int4 ch = chunks[c];
                    uint8_t* sb = smem + st * TC_STAGE_BYTES;
                    mbar_expect_tx(&sh->full[st], TC_STAGE_BYTES);
                    tma_load_2d(sb + 0 * TC_OPB, &map_hi, &sh->full[st], ch.x, rowA);
                    tma_load_2d(sb + 1 * TC_OPB, &map_lo, &sh->full[st], ch.x, rowA);
#pragma unroll
                    for (int q = 0; q < S::B_BOXES; ++q) {
                        tma_load_2d(sb + (2 + q) * TC_OPB, &map_hi, &sh->full[st], ch.y,
                                    rowB + 128 * q);
                        tma_load_2d(sb + (2 + S::B_BOXES + q) * TC_OPB, &map_lo, &sh->full[st],
                                    ch.y, rowB + 128 * q);
                    }
                }
            }
            if (*abort_flag) {   // let the copies already issued land before the CTA exits
                for (long long c = (gc > TC_STAGES ? gc - TC_STAGES : 0); c < gc; ++c)
                    if (c != withheld)
                        mbar_drain(&sh->full[c % TC_STAGES], (uint32_t)(c / TC_STAGES) & 1u,
                                   wait_limit);
            }
        }
    } else if (warp == EPI + 1) {
        // ---------------------------------------------------------------- MMA issuer
        if (lane == 0) {
            bool issued_any = false, stop = false;
            long long gc = 0, gg = 0;            // chunks and accumulation groups of this CTA
            for (int lt = 0; lt < my_tiles && !stop; ++lt) {
                int4 ch_next = chunks[0];        // schedule entry, read one chunk ahead
                for (int c = 0; c < nchunks; ++c, ++gc) {
                    const int4 ch = ch_next;
                    if (c + 1 < nchunks) ch_next = chunks[c + 1];
                    const int st = (int)(gc % TC_STAGES);
                    const uint32_t ph = (uint32_t)(gc / TC_STAGES) & 1u;
                    const int b = (int)(gg % NBUF);
                    const long long use = gg / NBUF;        // earlier uses of buffer b
                    const bool first = (c % gsize) == 0;
                    const bool last = ((c % gsize) == gsize - 1) || c == nchunks - 1;
                    if (first && use >= 1 &&
                        !mbar_wait(&sh->acc_empty[b], (uint32_t)((use - 1) & 1), abort_flag,
                                   status, wait_limit)) {
                        stop = true;
                        break;
                    }
                    if (!mbar_wait(&sh->full[st], ph, abort_flag, status, wait_limit)) {
                        stop = true;
                        break;
                    }
                    tc_fence_after();
                    const bool neg = ch.z != 0;             // r', s' blocks (chunk schedule)
                    const uint32_t idesc = neg ? IDESC_NEG : IDESC;
                    const uint32_t d = tmem + (uint32_t)(b * BN);
                    const uint32_t sa = smem_u32(smem + st * TC_STAGE_BYTES);
                    // three products per K step; the lo.lo product too for marked chunks (one
                    // branch per chunk, both bodies fully unrolled)
                    auto mma_chunk = [&](auto four) {
#pragma unroll
                        for (int k = 0; k < TC_BK / 16; ++k) {
                            const uint64_t ahi = sdesc_sw128(sa + 0 * TC_OPB + k * 32);
                            const uint64_t alo = sdesc_sw128(sa + 1 * TC_OPB + k * 32);
                            const uint64_t bhi = sdesc_sw128(sa + 2 * TC_OPB + k * 32);
                            const uint64_t blo =
                                sdesc_sw128(sa + (2 + S::B_BOXES) * TC_OPB + k * 32);
                            umma_bf16(d, ahi, bhi, idesc, (first && k == 0) ? 0u : 1u);
                            umma_bf16(d, ahi, blo, idesc, 1u);
                            umma_bf16(d, alo, bhi, idesc, 1u);
                            if (decltype(four)::value) umma_bf16(d, alo, blo, idesc, 1u);
                        }
                    };
                    if (LOLO || ch.w != 0)
                        mma_chunk(std::true_type{});
                    else
                        mma_chunk(std::false_type{});
                    issued_any = true;
                    umma_commit(&sh->empty[st]);
                    if (last) {
                        umma_commit(&sh->acc_full[b]);
                        ++gg;
                    }
                }
            }
            if (*abort_flag && issued_any) {   // wait for the MMAs in flight
                umma_commit(&sh->mma_done);
                mbar_drain(&sh->mma_done, 0, wait_limit);
            }
        }
    } else {
        // ---------------------------------------------------------------- epilogue
        const int q = warp & 3, h = warp >> 2;
        const int row = q * 32 + lane;
        bool ok = true;
        long long gg = 0;
        for (int lt = 0; lt < my_tiles && ok; ++lt) {
            const Tile t = tile_of(lt);
            float acc[EC], cmp[KAHAN ? EC : 1];
#pragma unroll
            for (int j = 0; j < EC; ++j) acc[j] = 0.f;
#pragma unroll
            for (int j = 0; j < (KAHAN ? EC : 1); ++j) cmp[j] = 0.f;
            for (int g = 0; g < ngroups; ++g, ++gg) {
                const int b = (int)(gg % NBUF);
                const long long use = gg / NBUF;
                ok = mbar_wait(&sh->acc_full[b], (uint32_t)(use & 1), abort_flag, status,
                               wait_limit);
                __syncwarp();
                ok = __all_sync(0xffffffffu, ok);
                if (!ok) break;
                tc_fence_after();
                const uint32_t taddr =
                    tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * BN + h * EC);
                // BN = 256 (16 epilogue warps, 112 registers each): 16-column loads, so that
                // the 64 running sums and the loaded columns fit without spilling
                constexpr int LDC = BN == 256 ? 16 : 32;
#pragma unroll
                for (int half = 0; half < EC / LDC; ++half) {
                    uint32_t r[LDC];
                    if constexpr (LDC == 16)
                        tmem_ld16(taddr + half * LDC, r);
                    else
                        tmem_ld32(taddr + half * LDC, r);
                    tmem_ld_wait();
#pragma unroll
                    for (int j = 0; j < LDC; ++j) {
                        const float x = __uint_as_float(r[j]);
                        float& s = acc[half * LDC + j];
                        if (KAHAN) {
                            float& c = cmp[KAHAN ? half * LDC + j : 0];
                            const float y = x - c;
                            const float tt = s + y;
                            c = (tt - s) - y;
                            s = tt;
                        } else {
                            s += x;
                        }
                    }
                }
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(&sh->acc_empty[b]);
            }
            if (!ok || *abort_flag) break;
            const PdDev pd = pds[t.pd];
            const double sc = (double)feature_scale_from_bits(scale_bits[t.pd]);
            const double inv_sc2 = 1.0 / (sc * sc);
            const int n = pd.n;
            const int gi = t.I * TC_M + row;
            double* Dp = D + pd.d_off;
            const double* an = pair_norm + pd.img_off;
            if (gi < n) {
                const double ai = an[gi];
                const int j0 = t.J * BN + h * EC;
#pragma unroll
                for (int j = 0; j < EC; ++j) {
                    const int gj = j0 + j;
                    // blocks of 8 columns: keeps the compiler from hoisting all 64 norm loads
                    // ahead of the stores (their registers would spill the running sums)
                    if ((j & 7) == 0) asm volatile("" ::: "memory");
                    if (gj >= n || gj < gi) continue;
                    if (gj == gi) {
                        Dp[(int64_t)gi * n + gi] = 0.0;
                        continue;
                    }
                    const float e = KAHAN ? (acc[j] - cmp[KAHAN ? j : 0]) : acc[j];
                    const double v = ai + an[gj] + (double)e * inv_sc2;
                    Dp[(int64_t)gi * n + gj] = v;
                    Dp[(int64_t)gj * n + gi] = v;
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == EPI + 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(TMEM_COLS)
                     : "memory");
    }
}

// ---- the CTA-pair form: 256 x 128 tiles on two SMs (cta_group::2) --------------------------
// A cluster of two CTAs on two SMs computes a 256 x 128 tile with one MMA stream: the even
// CTA issues tcgen05.mma.cta_group::2 (M = 256, N = 128); each CTA holds 128 rows of A and 64
// of the 128 B rows of every stage in its own shared memory, and 128 accumulator rows in its
// own tensor memory.  Per SM a 64-wide K chunk moves 48 KB (A 32 KB, half of B 16 KB) instead
// of the 64 KB of a 128 x 128 tile on one SM, and four stages fit in shared memory.
//   loads:  both CTAs' TMA copies count on the even CTA's full barrier (the even CTA arms it
//           with both CTAs' bytes);
//   MMA:    one thread of the even CTA; its commits arrive on the stage's empty barrier and
//           the accumulator's full barrier of both CTAs (multicast);
//   epilogue: each CTA drains its own tensor memory and arrives on the even CTA's
//           accumulator-empty barrier (16 arrivals per group).
// Waits are bounded as in the one-SM kernel.  After an abort the even CTA waits (bounded) for
// the stages it armed; the odd CTA, whose copies count on the even CTA's barriers, waits a
// bounded time far longer than a copy takes before both CTAs meet at the final cluster barrier.
constexpr int TP_STAGES = 4;
constexpr int TP_OPB_B = 64 * TC_BK * 2;                      // one 64-row box: 8 KB
constexpr int TP_STAGE_BYTES = 2 * TC_OPB + 2 * TP_OPB_B;      // 48 KB per CTA
constexpr size_t TP_SMEM = (size_t)TP_STAGES * TP_STAGE_BYTES + 1024 + 512;

struct TpShared {
    uint64_t full[TP_STAGES];
    uint64_t empty[TP_STAGES];
    uint64_t acc_full[TC_MAX_BUFS];
    uint64_t acc_empty[TC_MAX_BUFS];
    uint64_t mma_done;
    uint32_t tmem_base;
    int abort_flag;
};

template <bool LOLO, int NBUF>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(TC_THREADS, 1) gemm_tc_pair_kernel(
        const __grid_constant__ CUtensorMap map_hi, const __grid_constant__ CUtensorMap map_lo,
        const __grid_constant__ CUtensorMap mapb_hi, const __grid_constant__ CUtensorMap mapb_lo,
        const double* __restrict__ pair_norm, const uint32_t* __restrict__ scale_bits,
        const Tile* __restrict__ tiles, const PdDev* __restrict__ pds, double* __restrict__ D,
        uint32_t* __restrict__ status, const int4* __restrict__ chunks, int nchunks,
        int group_chunks, long long wait_limit, int withhold, int tile_begin, int tile_count) {
    static_assert(NBUF == 2 || NBUF == 4, "two or four TMEM accumulators");
    constexpr int BN = 128, EC = 64;
    constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                               ((uint32_t)(256 >> 4) << 24);
    constexpr uint32_t IDESC_NEG = IDESC | (1u << 14);
    constexpr uint32_t TMEM_COLS = NBUF * BN;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    TpShared* sh = (TpShared*)(smem + TP_STAGES * TP_STAGE_BYTES);
    volatile int* abort_flag = &sh->abort_flag;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t rank = cluster_ctarank();
    const bool even = rank == 0;
    const int pair = (int)(blockIdx.x >> 1), npairs = (int)(gridDim.x >> 1);
    const int my_tiles = pair < tile_count ? (tile_count - pair + npairs - 1) / npairs : 0;
    auto tile_of = [&](int lt) { return tiles[tile_begin + pair + lt * npairs]; };
    const int gsize = (group_chunks > 0 && group_chunks < nchunks) ? group_chunks : nchunks;
    const int ngroups = (nchunks + gsize - 1) / gsize;

    if (threadIdx.x == 0) {
        for (int s = 0; s < TP_STAGES; ++s) {
            mbar_init(&sh->full[s], 1);
            mbar_init(&sh->empty[s], 1);
        }
        for (int b = 0; b < NBUF; ++b) {
            mbar_init(&sh->acc_full[b], 1);
            mbar_init(&sh->acc_empty[b], 2 * TC_EPI_WARPS);
        }
        mbar_init(&sh->mma_done, 1);
        sh->abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == TC_EPI_WARPS + 1) {
        asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(&sh->tmem_base)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    cluster_sync();              // both CTAs' barriers and tensor memory are ready
    tc_fence_after();
    const uint32_t tmem = sh->tmem_base;
    // the even CTA's full and accumulator-empty barriers, as cluster addresses
    const uint32_t full_even = map_to_cta(smem_u32(&sh->full[0]), 0);
    const uint32_t acc_empty_even = map_to_cta(smem_u32(&sh->acc_empty[0]), 0);

    if (warp == TC_EPI_WARPS) {
        // ---------------------------------------------------------------- TMA producer
        if (lane == 0) {
            asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&map_hi) : "memory");
            asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&map_lo) : "memory");
            asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&mapb_hi) : "memory");
            asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&mapb_lo) : "memory");
            long long gc = 0, withheld = -1;
            bool stop = false;
            for (int lt = 0; lt < my_tiles && !stop; ++lt) {
                const Tile t = tile_of(lt);
                const PdDev pd = pds[t.pd];
                const int rowA = (int)(pd.row_off + (int64_t)t.I * 256 + rank * 128);
                const int rowB = (int)(pd.row_off + (int64_t)t.J * BN + rank * 64);
                for (int c = 0; c < nchunks; ++c, ++gc) {
                    const int st = (int)(gc % TP_STAGES);
                    const uint32_t ph = (uint32_t)(gc / TP_STAGES) & 1u;
                    if (gc >= TP_STAGES &&
                        !mbar_wait(&sh->empty[st], ph ^ 1u, abort_flag, status, wait_limit)) {
                        stop = true;
                        break;
                    }
                    if (lt == 0 && c == withhold) {      // test of the timeout path
                        withheld = gc;
                        continue;
                    }
                    const int4 ch = chunks[c];
                    uint8_t* sb = smem + st * TP_STAGE_BYTES;
                    if (even) mbar_expect_tx(&sh->full[st], 2 * TP_STAGE_BYTES);
                    const uint32_t bar = full_even + 8u * (uint32_t)st;
                    tma_load_2d_pair(sb, &map_hi, bar, ch.x, rowA);
                    tma_load_2d_pair(sb + TC_OPB, &map_lo, bar, ch.x, rowA);
                    tma_load_2d_pair(sb + 2 * TC_OPB, &mapb_hi, bar, ch.y, rowB);
                    tma_load_2d_pair(sb + 2 * TC_OPB + TP_OPB_B, &mapb_lo, bar, ch.y, rowB);
                }
            }
            if (*abort_flag) {
                if (even) {      // the stages this CTA armed: both CTAs' copies have landed
                    for (long long c = (gc > TP_STAGES ? gc - TP_STAGES : 0); c < gc; ++c)
                        if (c != withheld)
                            mbar_drain(&sh->full[c % TP_STAGES],
                                       (uint32_t)(c / TP_STAGES) & 1u, wait_limit);
                } else {         // copies count on the even CTA's barriers: a bounded pause
                    const long long t0 = clock64();
                    const long long pause = wait_limit < (1ll << 22) ? wait_limit : (1ll << 22);
                    while (clock64() - t0 < pause) __nanosleep(1000);
                }
            }
        }
    } else if (warp == TC_EPI_WARPS + 1) {
        // ---------------------------------------------------------------- MMA issuer
        if (lane == 0 && even) {
            bool issued_any = false, stop = false;
            long long gc = 0, gg = 0;
            for (int lt = 0; lt < my_tiles && !stop; ++lt) {
                int4 ch_next = chunks[0];
                for (int c = 0; c < nchunks; ++c, ++gc) {
                    const int4 ch = ch_next;
                    if (c + 1 < nchunks) ch_next = chunks[c + 1];
                    const int st = (int)(gc % TP_STAGES);
                    const uint32_t ph = (uint32_t)(gc / TP_STAGES) & 1u;
                    const int b = (int)(gg % NBUF);
                    const long long use = gg / NBUF;
                    const bool first = (c % gsize) == 0;
                    const bool last = ((c % gsize) == gsize - 1) || c == nchunks - 1;
                    if (first && use >= 1 &&
                        !mbar_wait(&sh->acc_empty[b], (uint32_t)((use - 1) & 1), abort_flag,
                                   status, wait_limit)) {
                        stop = true;
                        break;
                    }
                    if (!mbar_wait(&sh->full[st], ph, abort_flag, status, wait_limit)) {
                        stop = true;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t idesc = ch.z != 0 ? IDESC_NEG : IDESC;
                    const uint32_t d = tmem + (uint32_t)(b * BN);
                    const uint32_t sa = smem_u32(smem + st * TP_STAGE_BYTES);
                    auto mma_chunk = [&](auto four) {
#pragma unroll
                        for (int k = 0; k < TC_BK / 16; ++k) {
                            const uint64_t ahi = sdesc_sw128(sa + k * 32);
                            const uint64_t alo = sdesc_sw128(sa + TC_OPB + k * 32);
                            const uint64_t bhi = sdesc_sw128(sa + 2 * TC_OPB + k * 32);
                            const uint64_t blo = sdesc_sw128(sa + 2 * TC_OPB + TP_OPB_B + k * 32);
                            umma_bf16_pair(d, ahi, bhi, idesc, (first && k == 0) ? 0u : 1u);
                            umma_bf16_pair(d, ahi, blo, idesc, 1u);
                            umma_bf16_pair(d, alo, bhi, idesc, 1u);
                            if (decltype(four)::value) umma_bf16_pair(d, alo, blo, idesc, 1u);
                        }
                    };
                    if (LOLO || ch.w != 0)
                        mma_chunk(std::true_type{});
                    else
                        mma_chunk(std::false_type{});
                    issued_any = true;
                    umma_commit_pair(&sh->empty[st], (uint16_t)3);
                    if (last) {
                        umma_commit_pair(&sh->acc_full[b], (uint16_t)3);
                        ++gg;
                    }
                }
            }
            if (*abort_flag && issued_any) {   // wait for the MMAs in flight
                umma_commit_pair(&sh->mma_done, (uint16_t)1);
                mbar_drain(&sh->mma_done, 0, wait_limit);
            }
        }
    } else {
        // ---------------------------------------------------------------- epilogue
        const int q = warp & 3, h = warp >> 2;
        const int row = q * 32 + lane;
        bool ok = true;
        long long gg = 0;
        for (int lt = 0; lt < my_tiles && ok; ++lt) {
            const Tile t = tile_of(lt);
            float acc[EC];
#pragma unroll
            for (int j = 0; j < EC; ++j) acc[j] = 0.f;
            for (int g = 0; g < ngroups; ++g, ++gg) {
                const int b = (int)(gg % NBUF);
                const long long use = gg / NBUF;
                ok = mbar_wait(&sh->acc_full[b], (uint32_t)(use & 1), abort_flag, status,
                               wait_limit);
                __syncwarp();
                ok = __all_sync(0xffffffffu, ok);
                if (!ok) break;
                tc_fence_after();
                const uint32_t taddr =
                    tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * BN + h * EC);
#pragma unroll
                for (int half = 0; half < EC / 32; ++half) {
                    uint32_t r[32];
                    tmem_ld32(taddr + half * 32, r);
                    tmem_ld_wait();
#pragma unroll
                    for (int j = 0; j < 32; ++j) acc[half * 32 + j] += __uint_as_float(r[j]);
                }
                tc_fence_before();
                __syncwarp();
                // the accumulator's columns are in registers (tcgen05.wait::ld above): a relaxed
                // arrive suffices, and a release at cluster scope cost a memory barrier per
                // warp and group (the kernel's top stall)
                if (lane == 0) mbar_arrive_cluster_relaxed(acc_empty_even + 8u * (uint32_t)b);
            }
            if (!ok || *abort_flag) break;
            const PdDev pd = pds[t.pd];
            const double sc = (double)feature_scale_from_bits(scale_bits[t.pd]);
            const double inv_sc2 = 1.0 / (sc * sc);
            const int n = pd.n;
            const int gi = t.I * 256 + (int)rank * 128 + row;
            double* Dp = D + pd.d_off;
            const double* an = pair_norm + pd.img_off;
            if (gi < n) {
                const double ai = an[gi];
                const int j0 = t.J * BN + h * EC;
#pragma unroll
                for (int j = 0; j < EC; ++j) {
                    const int gj = j0 + j;
                    if (gj >= n || gj < gi) continue;
                    if (gj == gi) {
                        Dp[(int64_t)gi * n + gi] = 0.0;
                        continue;
                    }
                    const double v = ai + an[gj] + (double)acc[j] * inv_sc2;
                    Dp[(int64_t)gi * n + gj] = v;
                    Dp[(int64_t)gj * n + gi] = v;
                }
            }
        }
    }
    tc_fence_before();
    cluster_sync();              // the pair's MMAs, copies and remote arrivals are done
    if (warp == TC_EPI_WARPS + 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(TMEM_COLS)
                     : "memory");
    }
}

}  // namespace

namespace kern {
int gemm_split_bf16(const mem_plan& P, const void* feat_hi, const void* feat_lo,
                    const double* pair_norm, const uint32_t* scale_bits, const Tile* tiles,
                    const PdDev* pds, const int4* chunks, double* D, uint32_t* status,
                    cudaStream_t s) {
    if (P.tiles.empty() || !D) return MEM_OK;
    // every chunk starts on a 64-column boundary: TMA x offsets are multiples of 8 bf16
    if (P.Kf % TC_BK != 0 || P.n_rows % TC_M != 0 || (int64_t)P.n_chunks * TC_BK != P.Kf)
        return MEM_ERR_INVALID;
    CUtensorMap mhi, mlo;
    int st = tc::make_map(&mhi, feat_hi, P.Kf, P.n_rows);
    if (st != MEM_OK) return st;
    st = tc::make_map(&mlo, feat_lo, P.Kf, P.n_rows);
    if (st != MEM_OK) return st;
    const int sms = P.num_sms > 0 ? P.num_sms : 1;
    CUtensorMap bhi, blo;                // 64-row boxes: the CTA pairs' halves of B
    bool have_b64 = false;
    // one launch per size class of the plan's contraction configuration (tiles sorted by class)
    for (size_t k = 0; k < P.tc_ranges.size(); ++k) {
        const int begin = P.tc_ranges[k].first, count = P.tc_ranges[k].second;
        if (count <= 0) continue;
        const mem_contraction_config& cfg = P.tc_classes[k];
        if (cfg.tile_m == 256) {
            if (!have_b64) {
                st = tc::make_map(&bhi, feat_hi, P.Kf, P.n_rows, 64);
                if (st != MEM_OK) return st;
                st = tc::make_map(&blo, feat_lo, P.Kf, P.n_rows, 64);
                if (st != MEM_OK) return st;
                have_b64 = true;
            }
            const unsigned pgrid =
                2u * (unsigned)(cfg.persistent ? std::min(count, std::max(1, sms / 2)) : count);
#define MEM_TP_LAUNCH(LOLO, NB)                                                                \
    do {                                                                                       \
        MEM_CUDA_TRY(cudaFuncSetAttribute(gemm_tc_pair_kernel<LOLO, NB>,                       \
                                          cudaFuncAttributeMaxDynamicSharedMemorySize,         \
                                          (int)TP_SMEM));                                      \
        gemm_tc_pair_kernel<LOLO, NB><<<pgrid, TC_THREADS, TP_SMEM, s>>>(                      \
            mhi, mlo, bhi, blo, pair_norm, scale_bits, tiles, pds, D, status, chunks,          \
            P.n_chunks, P.tc_group_chunks, P.wait_cycles, P.test_withhold_chunk, begin,        \
            count);                                                                            \
    } while (0)
            if (P.tc_lolo) {
                if (cfg.accumulators == 4) MEM_TP_LAUNCH(true, 4); else MEM_TP_LAUNCH(true, 2);
            } else {
                if (cfg.accumulators == 4) MEM_TP_LAUNCH(false, 4); else MEM_TP_LAUNCH(false, 2);
            }
#undef MEM_TP_LAUNCH
            MEM_LAUNCH_CHECK();
            continue;
        }
        const unsigned grid = cfg.persistent ? (unsigned)std::min(count, sms) : (unsigned)count;
#define MEM_TC_LAUNCH(KAHAN, LOLO, NB, BN)                                                     \
    do {                                                                                       \
        MEM_CUDA_TRY(cudaFuncSetAttribute(gemm_tc_kernel<KAHAN, LOLO, NB, BN>,                 \
                                          cudaFuncAttributeMaxDynamicSharedMemorySize,         \
                                          (int)TcShape<BN>::SMEM));                            \
        gemm_tc_kernel<KAHAN, LOLO, NB, BN><<<grid, TcShape<BN>::THREADS, TcShape<BN>::SMEM,   \
                                              s>>>(                                            \
            mhi, mlo, pair_norm, scale_bits, tiles, pds, D, status, chunks, P.n_chunks,        \
            P.tc_group_chunks, P.wait_cycles, P.test_withhold_chunk, begin, count);            \
    } while (0)
#define MEM_TC_SHAPE(KAHAN, LOLO)                                                              \
    do {                                                                                       \
        if (cfg.tile_n == 256) MEM_TC_LAUNCH(KAHAN, LOLO, 2, 256);                             \
        else if (cfg.accumulators == 4) MEM_TC_LAUNCH(KAHAN, LOLO, 4, 128);                    \
        else MEM_TC_LAUNCH(KAHAN, LOLO, 2, 128);                                               \
    } while (0)
        // the compensated sums of the 256-wide tile would not fit the register file: its
        // classes keep the 128-wide kernel (apply_contraction) when MEM_TC_KAHAN is set
        if (P.tc_kahan) {
            if (P.tc_lolo) MEM_TC_LAUNCH(true, true, 2, 128); else MEM_TC_LAUNCH(true, false, 2, 128);
        } else {
            if (P.tc_lolo) MEM_TC_SHAPE(false, true); else MEM_TC_SHAPE(false, false);
        }
#undef MEM_TC_SHAPE
#undef MEM_TC_LAUNCH
        MEM_LAUNCH_CHECK();
    }
    return MEM_OK;
}
}  // namespace kern
}  // namespace mem
