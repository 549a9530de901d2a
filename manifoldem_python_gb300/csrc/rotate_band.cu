// The two periodic cubic B-spline rotations of rotatefill.op (modules/rotatefill.py:21-41,
// called at modules/getDistanceCTF_local_Conj9combinedS2.py:328-330) for boxes whose
// coefficient image does not fit one CTA's shared memory (64 < N <= 512 without a compile-time
// kernel; N = 250 is the 1500-PD workload's box).  One CTA of 512 threads per image.
//
// Each rotation is split where the separable prefilter splits:
//   1. the prefilter along layout columns (every line runs across all N layout rows), from the
//      input image in global memory to the image's scratch slot A: lanes on 32 consecutive
//      columns, each thread's 32-sample segment of a column in registers (coalesced loads and
//      stores, one L2 round trip per sample);
//   2. for each band of H0 consecutive layout rows (plus the 3-row periodic halo of the 4x4
//      window): the band's rows from A into shared memory, the prefilter along each row there
//      (complete lines), the 3-column periodic halo, and every output sample whose window
//      starts in the band, written straight to its output pixel.
// The first rotation reads the low-passed image in its storage orientation (transposed), so its
// layout rows are reference columns: it samples at (Y, X) and filters the reference rows first,
// as the other rotation kernels do.  The second rotation reads the first one's output in the
// reference orientation.  Outputs (and the second rotation's input) are reference-oriented.
#include <cmath>

#include "mem_internal.cuh"
#include "rotate_fixed.cuh"

namespace mem {
namespace {

using rot::kZ1;
using rot::mask_ref;
using rot::RotConst;

constexpr int kBandThreads = 512;
constexpr int kBandSeg = 32;                  // prefilter segment held in registers
constexpr int kMaxBandN = kBandThreads;       // one output row per thread per pass at most

__device__ __forceinline__ int wrap_n(int i, int N) {      // i in [-N, 2N) -> [0, N)
    i += (i < 0) ? N : 0;
    return i - ((i >= N) ? N : 0);
}

// One periodic prefilter pass over `lines` lines of N samples, split into nsg segments of
// kBandSeg samples (the last one N - 32 (nsg - 1) long), one thread per segment with the
// segment in registers.  Lines go in rounds of LPR = 32 floor(NT / (32 nsg)), a warp holding
// one segment of 32 consecutive lines.  Causal pass c+[k] = x[k] + z1 c+[k-1]: each thread
// forms its segment's end state from zero, E_g = sum_k z1^(L_g - 1 - k) x[k], and starts its
// recursion from E_{g-1} + z1^L_{g-1} E_{g-2} (periodic in g; the omitted terms are below
// z1^58 = 6e-34 of the state).  The anticausal pass c-[k] = c+[k] + z1 c-[k+1] does the same
// from the right, and the output is -6 z1 c-[k].  load(l, k) gives sample k of line l,
// store(l, k, v) takes the result; carry holds 2 NT floats.  Ends with a barrier.
template <int NT, class Load, class Store>
__device__ __forceinline__ void prefilter_lines(int lines, int N, int nsg, float zlast,
                                                float* carry, Load load, Store store) {
    constexpr float zseg = rot::z1_pow<kBandSeg>();
    constexpr float gain = -6.0f * kZ1;
    const int lpr = 32 * (NT / (32 * nsg));
    const int t = threadIdx.x;
    const int lw = t % lpr, g = t / lpr;
    const bool has_seg = g < nsg;
    const int k0 = g * kBandSeg;
    const int len = has_seg ? min(kBandSeg, N - k0) : 0;
    float* carry_c = carry;              // [nsg][lpr] causal end states
    float* carry_a = carry + NT;         // [nsg][lpr] anticausal start states
    const int g1 = g == 0 ? nsg - 1 : g - 1, g2 = g1 == 0 ? nsg - 1 : g1 - 1;
    const int h1 = g == nsg - 1 ? 0 : g + 1, h2 = h1 == nsg - 1 ? 0 : h1 + 1;
    const float zg1 = g1 == nsg - 1 ? zlast : zseg;
    const float zh1 = h1 == nsg - 1 ? zlast : zseg;
    for (int l0 = 0; l0 < lines; l0 += lpr) {
        const int l = l0 + lw;
        const bool active = has_seg && l < lines;
        float v[kBandSeg];
        if (active) {
            float e = 0.f;
#pragma unroll
            for (int k = 0; k < kBandSeg; ++k) {
                if (k < len) {
                    v[k] = load(l, k0 + k);
                    e = fmaf(kZ1, e, v[k]);
                }
            }
            carry_c[g * lpr + lw] = e;
        }
        __syncthreads();
        if (active) {
            float c = fmaf(zg1, carry_c[g2 * lpr + lw], carry_c[g1 * lpr + lw]);
#pragma unroll
            for (int k = 0; k < kBandSeg; ++k) {
                if (k < len) {
                    c = fmaf(kZ1, c, v[k]);
                    v[k] = c;
                }
            }
            float e = 0.f;
#pragma unroll
            for (int k = kBandSeg - 1; k >= 0; --k)
                if (k < len) e = fmaf(kZ1, e, v[k]);
            carry_a[g * lpr + lw] = e;
        }
        __syncthreads();
        if (active) {
            float c = fmaf(zh1, carry_a[h2 * lpr + lw], carry_a[h1 * lpr + lw]);
#pragma unroll
            for (int k = kBandSeg - 1; k >= 0; --k) {
                if (k < len) {
                    c = fmaf(kZ1, c, v[k]);
                    store(l, k0 + k, gain * c);
                }
            }
        }
        __syncthreads();
    }
}

// One output sample from the band: layout coordinates (U, V) in 32.32 fixed point with the
// window's -1 folded in, band row rho = the window's first layout row - b0.
__device__ __forceinline__ float sample_band(const float* s, int P, int rho, int iv, int64_t U,
                                             int64_t V) {
    const float tu = (float)(uint32_t)(U & 0xffffffffll) * 2.3283064365386963e-10f;
    const float tv = (float)(uint32_t)(V & 0xffffffffll) * 2.3283064365386963e-10f;
    float wu[4], wv[4];
    rot::bspline_w(tu, wu);
    rot::bspline_w(tv, wv);
    const float* b = s + rho * P + iv;
    float acc = 0.f;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        float r = wv[0] * b[i * P];
        r = fmaf(wv[1], b[i * P + 1], r);
        r = fmaf(wv[2], b[i * P + 2], r);
        r = fmaf(wv[3], b[i * P + 3], r);
        acc = fmaf(wu[i], r, acc);
    }
    return acc;
}

// One rotation: the layout-column prefilter from `in` to A, then the bands.  TRANS: `in` is
// transposed (layout row u = reference column), masked with the annular mask on load.
template <int NT, bool TRANS>
__device__ __forceinline__ void rotate_banded(const float* in, float* A, float* out, float* s,
                                              float* carry, const RotConst& Q, int N, int P,
                                              int H0, int nb, int nsg, float zlast) {
    // 1. along layout columns: line = column v, sample k = row u
    prefilter_lines<NT>(
        N, N, nsg, zlast, carry,
        [&](int v, int u) {
            const float x = __ldcg(in + (int64_t)u * N + v);
            return TRANS ? x * mask_ref(v, u, N) : x;
        },
        [&](int v, int u, float x) { A[(int64_t)u * N + v] = x; });
    constexpr int64_t kOne = 1ll << 32;
    const int R = NT / N;
    const int c = threadIdx.x % N, r0 = threadIdx.x / N;
    for (int b = 0; b < nb; ++b) {
        const int b0 = b * H0, h = min(H0, N - b0), rows = h + 3;
        // 2a. band rows b0 .. b0 + h + 2 (mod N) of A, a warp per row
        for (int rho = threadIdx.x >> 5; rho < rows; rho += NT / 32) {
            const float* src = A + (int64_t)wrap_n(b0 + rho, N) * N;
            float* dst = s + rho * P;
            for (int v = threadIdx.x & 31; v < N; v += 32) dst[v] = __ldcg(src + v);
        }
        __syncthreads();
        // 2b. along layout rows, in shared memory (lanes on consecutive rows: the row stride is
        // 1 mod 32, so a warp's 32 accesses fall in 32 banks)
        prefilter_lines<NT>(
            rows, N, nsg, zlast, carry, [&](int rho, int v) { return s[rho * P + v]; },
            [&](int rho, int v, float x) { s[rho * P + v] = x; });
        for (int p = threadIdx.x; p < rows * 3; p += NT) {
            const int rho = p / 3, j = p - rho * 3;
            s[rho * P + N + j] = s[rho * P + j];
        }
        __syncthreads();
        // 2c. every output whose window starts in the band.  Thread (c, r0) owns rows
        // r0 + j R, j < J; along them the window's first layout row U_j = U_0 + j dU is linear,
        // so the rows in the band (its rows b0 .. b0 + h - 1, met as U in [b0, b0 + h) + k N,
        // k = -1, 0, 1, since U stays within (-N, 2N)) are up to three ranges of j, found from
        // U_0 and dU (widened by one step each way; each sample still checks its row).
        if (r0 < R) {
            const int64_t X0 = Q.bx - kOne + (int64_t)r0 * Q.rc + (int64_t)c * Q.rs;
            const int64_t Y0 = Q.by - kOne - (int64_t)r0 * Q.rs + (int64_t)c * Q.rc;
            const int64_t dX = (int64_t)R * Q.rc, dY = -(int64_t)R * Q.rs;
            const int64_t U0 = TRANS ? Y0 : X0, dU = TRANS ? dY : dX;
            const int J = (N - r0 + R - 1) / R;
            for (int k = -1; k <= 1; ++k) {
                int j0 = 0, j1 = J;
                if (dU != 0) {
                    // in units of rows of the layout: U_0 / 2^32 and dU / 2^32 (float is exact
                    // enough: the range is widened by a step each way)
                    const float u0 = (float)U0 * 2.3283064365386963e-10f;
                    const float inv = 4294967296.0f / (float)dU;
                    const float a = ((float)(b0 + k * N) - u0) * inv;
                    const float e = ((float)(b0 + h + k * N) - u0) * inv;
                    const float lo = fminf(fmaxf(fminf(a, e), -2.f), (float)J + 2.f);
                    const float hi = fminf(fmaxf(fmaxf(a, e), -2.f), (float)J + 2.f);
                    j0 = max(0, (int)floorf(lo) - 1);
                    j1 = min(J, (int)ceilf(hi) + 1);
                } else if (k != 0) {
                    continue;                      // a constant U: one pass over all rows
                }
                int64_t X = X0 + (int64_t)j0 * dX, Y = Y0 + (int64_t)j0 * dY;
                for (int j = j0; j < j1; ++j, X += dX, Y += dY) {
                    const int64_t U = TRANS ? Y : X, V = TRANS ? X : Y;
                    const int f = (int)(U >> 32);
                    const int rho = f - b0 - k * N;
                    if (dU == 0 ? (unsigned)(wrap_n(f, N) - b0) >= (unsigned)h
                                : (unsigned)rho >= (unsigned)h)
                        continue;
                    out[(int64_t)(r0 + j * R) * N + c] =
                            sample_band(s, P, dU == 0 ? wrap_n(f, N) - b0 : rho,
                                        wrap_n((int)(V >> 32), N), U, V);
                }
            }
        }
        __syncthreads();
    }
}

// xbuf: the low-passed image (storage orientation), then the first rotation's output; A: the
// image's spectrum slot (>= N^2 floats, free at this point) as coefficient scratch.
template <int NT>
__global__ void __launch_bounds__(NT, 2) rotate_band_kernel(
        float* xbuf, float2* spec, int64_t Kc, float* img_out, const RotConst* __restrict__ rotc,
        int N, int P, int H0, int nb, int nsg, float zlast) {
    extern __shared__ float sm[];
    float* carry = sm;                   // 2 NT floats
    float* s = sm + 2 * NT;              // (H0 + 3) x P band
    const int64_t img = blockIdx.x;
    const int64_t NN = (int64_t)N * N;
    float* B = xbuf + img * NN;
    float* A = reinterpret_cast<float*>(spec + img * Kc);
    const RotConst Q1 = rotc[2 * img], Q2 = rotc[2 * img + 1];
    // B is read by the first column pass before any band writes it
    rotate_banded<NT, true>(B, A, B, s, carry, Q1, N, P, H0, nb, nsg, zlast);
    rotate_banded<NT, false>(B, A, img_out + img * NN, s, carry, Q2, N, P, H0, nb, nsg, zlast);
}

}  // namespace

namespace kern {

bool rotate_band_supported(int N) { return N >= 64 && N <= kMaxBandN; }

int rotate_band(const mem_plan& P, float* xbuf, float2* spec, float* img_out, const void* rotc,
                cudaStream_t s) {
    if (P.n_images == 0) return MEM_OK;
    const int N = P.N;
    if (!rotate_band_supported(N) || P.Kc * 2 < (int64_t)N * N) return MEM_ERR_UNSUPPORTED;
    constexpr int NT = kBandThreads;
    const int Pst = ((N + 3 + 30) / 32) * 32 + 1;            // >= N + 3, = 1 mod 32
    // bands: the fewest whose shared memory lets two CTAs share an SM (MEM_ROT_BANDS overrides)
    const size_t budget = 100 * 1024 - 2 * NT * sizeof(float);
    int nb = 1;
    while ((size_t)((N + nb - 1) / nb + 3) * Pst * sizeof(float) > budget) ++nb;
    if (const char* e = std::getenv("MEM_ROT_BANDS")) nb = std::max(nb, std::atoi(e));
    const int H0 = (N + nb - 1) / nb;
    nb = (N + H0 - 1) / H0;
    const int nsg = (N + kBandSeg - 1) / kBandSeg;
    const int last = N - kBandSeg * (nsg - 1);
    const float zlast = (float)std::pow((double)kZ1, (double)last);
    const size_t smem = (2 * NT + (size_t)(H0 + 3) * Pst) * sizeof(float);
    if (smem > 227 * 1024) return MEM_ERR_UNSUPPORTED;
    MEM_CUDA_TRY(cudaFuncSetAttribute(rotate_band_kernel<NT>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    rotate_band_kernel<NT><<<(unsigned)P.n_images, NT, smem, s>>>(
            xbuf, spec, P.Kc, img_out, static_cast<const RotConst*>(rotc), N, Pst, H0, nb, nsg,
            zlast);
    MEM_LAUNCH_CHECK();
    return MEM_OK;
}

}  // namespace kern
}  // namespace mem
