// Plain FP32 form of the all-pairs CTF distance (reference :391-397):
//   D_ij = a_i + a_j + E_ij,   E_ij = u'_i.v'_j + v'_i.u'_j - r'_i.r'_j - s'_i.s'_j
// over the centred half-plane features written by features_kernel (prologue.cu).
// One CTA per upper-triangle 128 x 128 tile of a PD; 256 threads, 8 x 8 outputs per thread,
// FP32 FFMA accumulation, FP64 epilogue, mirrored store (D exactly symmetric, zero diagonal).
#include "mem_internal.cuh"

namespace mem {
namespace {

constexpr int TM = 128, TN = 128, BK = 16, NT = 256, APAD = 4;

__global__ void __launch_bounds__(NT) gemm_fp32_kernel(
        const float* __restrict__ X, const double* __restrict__ pair_norm,
        const uint32_t* __restrict__ scale_bits, const Tile* __restrict__ tiles,
        const PdDev* __restrict__ pds, const int4* __restrict__ chunks, double* __restrict__ D,
        int64_t Kf) {
    __shared__ __align__(16) float As[2][BK][TM + APAD];
    __shared__ __align__(16) float Bs[2][BK][TN + APAD];
    const Tile t = tiles[blockIdx.x];
    const PdDev pd = pds[t.pd];
    const int64_t K4 = Kf;
    const int tid = threadIdx.x;
    const int lrow = tid >> 2, lk = (tid & 3) * 4;
    const float* Abase = X + (pd.row_off + (int64_t)t.I * TM) * K4;
    const float* Bbase = X + (pd.row_off + (int64_t)t.J * TN) * K4;
    const int64_t nstage = K4 / BK;

    // stage st is the 16-column slice (st & 3) of 64-wide chunk st >> 2 of the plan's chunk
    // schedule (A column, B column, sign), which interleaves the feature blocks so that the
    // dominant low-frequency columns are accumulated last
    auto acol = [&](int64_t st) -> int64_t { return chunks[st >> 2].x + (st & 3) * BK; };
    auto bcol = [&](int64_t st) -> int64_t { return chunks[st >> 2].y + (st & 3) * BK; };

    float4 ra[2], rb[2];
    auto gload = [&](int64_t st) {
        const int64_t ka = acol(st);
        const int64_t kb = bcol(st);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int r = lrow + h * 64;
            ra[h] = *reinterpret_cast<const float4*>(Abase + (int64_t)r * K4 + ka + lk);
            rb[h] = *reinterpret_cast<const float4*>(Bbase + (int64_t)r * K4 + kb + lk);
        }
    };
    auto sstore = [&](int buf, int64_t st) {
        const float sg = chunks[st >> 2].z ? -1.0f : 1.0f;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int r = lrow + h * 64;
            As[buf][lk + 0][r] = sg * ra[h].x;
            As[buf][lk + 1][r] = sg * ra[h].y;
            As[buf][lk + 2][r] = sg * ra[h].z;
            As[buf][lk + 3][r] = sg * ra[h].w;
            Bs[buf][lk + 0][r] = rb[h].x;
            Bs[buf][lk + 1][r] = rb[h].y;
            Bs[buf][lk + 2][r] = rb[h].z;
            Bs[buf][lk + 3][r] = rb[h].w;
        }
    };

    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;

    const int ty = tid >> 4, tx = tid & 15;
    gload(0);
    sstore(0, 0);
    __syncthreads();
    for (int64_t st = 0; st < nstage; ++st) {
        const int buf = (int)(st & 1);
        if (st + 1 < nstage) gload(st + 1);
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            const float4 a0 = *reinterpret_cast<const float4*>(&As[buf][kk][ty * 4]);
            const float4 a1 = *reinterpret_cast<const float4*>(&As[buf][kk][64 + ty * 4]);
            const float4 b0 = *reinterpret_cast<const float4*>(&Bs[buf][kk][tx * 4]);
            const float4 b1 = *reinterpret_cast<const float4*>(&Bs[buf][kk][64 + tx * 4]);
            const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
            const float b[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
            for (int i = 0; i < 8; ++i)
#pragma unroll
                for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        if (st + 1 < nstage) {
            sstore(buf ^ 1, st + 1);
            __syncthreads();
        }
    }

    // epilogue: D = a_i + a_j + E / scale^2 in FP64, upper triangle + mirror
    const double sc = (double)feature_scale_from_bits(scale_bits[t.pd]);
    const double inv_sc2 = 1.0 / (sc * sc);
    const int n = pd.n;
    double* Dp = D + pd.d_off;
    const double* an = pair_norm + pd.img_off;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int gi = t.I * TM + (i < 4 ? ty * 4 + i : 64 + ty * 4 + i - 4);
        if (gi >= n) continue;
        const double ai = an[gi];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int gj = t.J * TN + (j < 4 ? tx * 4 + j : 64 + tx * 4 + j - 4);
            if (gj >= n || gj < gi) continue;
            if (gj == gi) {
                Dp[(int64_t)gi * n + gi] = 0.0;
                continue;
            }
            const double v = ai + an[gj] + (double)acc[i][j] * inv_sc2;
            Dp[(int64_t)gi * n + gj] = v;
            Dp[(int64_t)gj * n + gi] = v;
        }
    }
}

}  // namespace

namespace kern {
int gemm_fp32(const mem_plan& P, const float* feat, const double* pair_norm,
              const uint32_t* scale_bits, const Tile* tiles, const PdDev* pds,
              const int4* chunks, double* D, cudaStream_t s) {
    if (P.tiles.empty() || !D) return MEM_OK;
    if ((int64_t)P.n_chunks * 64 != P.Kf) return MEM_ERR_INVALID;
    gemm_fp32_kernel<<<(unsigned)P.tiles.size(), NT, 0, s>>>(feat, pair_norm, scale_bits, tiles, pds,
                                                             chunks, D, P.Kf);
    MEM_LAUNCH_CHECK();
    return MEM_OK;
}
}  // namespace kern
}  // namespace mem
