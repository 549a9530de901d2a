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
#include <cuda.h>
#include <type_traits>
#include <cudaTypedefs.h>

#include "mem_internal.cuh"

namespace mem {
namespace {

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
    static_assert(STAGES <= TC_MAX_STAGES, "stage ring");
};

// instruction descriptor, kind::f16: D f32 (bits 4-5 = 1), A bf16 (7-9 = 1), B bf16 (10-12 = 1),
// K-major A and B (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at bits 24-28, negate B bit 14
template <int BN>
__host__ __device__ constexpr uint32_t idesc_f16() {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
           ((uint32_t)(TC_M >> 4) << 24);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// bounded wait (at most `limit` SM clock cycles); false if it expired or another role aborted
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag,
                                          uint32_t* status, long long limit) {
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity)) {
        if (*abort_flag) return false;
        if (clock64() - t0 > limit) {
            *abort_flag = 1;
            atomicOr(status, kStatusTimeout);
            return false;
        }
    }
    return true;
}

// bounded wait used while draining after an abort (no abort check)
__device__ __forceinline__ void mbar_drain(uint64_t* bar, uint32_t parity, long long limit) {
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity))
        if (clock64() - t0 > limit) return;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar,
                                            int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
        "l"((uint64_t)map), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups 1024 B apart
__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t saddr) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)1 << 16;                  // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;        // stride byte offset
    d |= (uint64_t)1 << 46;                  // descriptor version
    d |= (uint64_t)2 << 61;                  // SWIZZLE_128B
    return d;
}

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                          uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t* bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
          "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
          "=r"(r[31])
        : "r"(taddr)
        : "memory");
}

__device__ __forceinline__ void tmem_ld_wait() {
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
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
__global__ void __launch_bounds__(TC_THREADS, 1) gemm_tc_kernel(
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
    constexpr int EC = BN / 2;                     // epilogue columns per thread
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
            mbar_init(&sh->acc_empty[b], TC_EPI_WARPS);
        }
        mbar_init(&sh->mma_done, 1);
        sh->abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == TC_EPI_WARPS + 1) {
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

    if (warp == TC_EPI_WARPS) {
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
    } else if (warp == TC_EPI_WARPS + 1) {
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
#pragma unroll
                for (int half = 0; half < EC / 32; ++half) {
                    uint32_t r[32];
                    tmem_ld32(taddr + half * 32, r);
                    tmem_ld_wait();
#pragma unroll
                    for (int j = 0; j < 32; ++j) {
                        const float x = __uint_as_float(r[j]);
                        float& s = acc[half * 32 + j];
                        if (KAHAN) {
                            float& c = cmp[KAHAN ? half * 32 + j : 0];
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
    if (warp == TC_EPI_WARPS + 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(TMEM_COLS)
                     : "memory");
    }
}

PFN_cuTensorMapEncodeTiled_v12000 get_encode() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    }
    return fn;
}

int make_map(CUtensorMap* map, const void* base, int64_t Kf, int64_t rows) {
    auto enc = get_encode();
    if (!enc) return MEM_ERR_CUDA;
    cuuint64_t dims[2] = {(cuuint64_t)Kf, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)(Kf * 2)};
    cuuint32_t box[2] = {(cuuint32_t)TC_BK, (cuuint32_t)TC_M};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims,
                     strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                     CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? MEM_OK : MEM_ERR_CUDA;
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
    int st = make_map(&mhi, feat_hi, P.Kf, P.n_rows);
    if (st != MEM_OK) return st;
    st = make_map(&mlo, feat_lo, P.Kf, P.n_rows);
    if (st != MEM_OK) return st;
    const int sms = P.num_sms > 0 ? P.num_sms : 1;
    // one launch per size class of the plan's contraction configuration (tiles sorted by class)
    for (size_t k = 0; k < P.tc_ranges.size(); ++k) {
        const int begin = P.tc_ranges[k].first, count = P.tc_ranges[k].second;
        if (count <= 0) continue;
        const mem_contraction_config& cfg = P.tc_classes[k];
        const unsigned grid = cfg.persistent ? (unsigned)std::min(count, sms) : (unsigned)count;
#define MEM_TC_LAUNCH(KAHAN, LOLO, NB, BN)                                                     \
    do {                                                                                       \
        MEM_CUDA_TRY(cudaFuncSetAttribute(gemm_tc_kernel<KAHAN, LOLO, NB, BN>,                 \
                                          cudaFuncAttributeMaxDynamicSharedMemorySize,         \
                                          (int)TcShape<BN>::SMEM));                            \
        gemm_tc_kernel<KAHAN, LOLO, NB, BN><<<grid, TC_THREADS, TcShape<BN>::SMEM, s>>>(       \
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
