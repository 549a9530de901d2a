// The two periodic cubic B-spline rotations of rotatefill.op (modules/rotatefill.py:21-41,
// called at modules/getDistanceCTF_local_Conj9combinedS2.py:328-330) for boxes whose
// coefficient image does not fit one CTA's shared memory (64 < N <= 512 without a compile-time
// kernel; N = 250 is the 1500-PD workload's box).  One CTA per image (512 threads, one CTA per
// SM, by default; the launcher's variants are described at rotate_band).
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

// The three phases of one segment's prefilter (see prefilter_lines).  FULL: the segment has
// kBandSeg samples (no per-sample length checks), else len < kBandSeg.  Sample k of the
// segment is in[k * ks] (times the annular mask at (mrow, mcol0 + k) when MASK); GLOBAL: `in`
// is global memory written earlier in this kernel (read through L2), else shared memory.
template <bool FULL, bool GLOBAL, bool MASK>
__device__ __forceinline__ float seg_causal_end(float* v, int len, const float* in, int ks,
                                                int N, int mrow, int mcol0) {
    float e = 0.f;
#pragma unroll
    for (int k = 0; k < kBandSeg; ++k) {
        if (FULL || k < len) {
            const float x = GLOBAL ? __ldcg(in) : *in;
            v[k] = MASK ? x * mask_ref(mrow, mcol0 + k, N) : x;
            e = fmaf(kZ1, e, v[k]);
            in += ks;
        }
    }
    return e;
}

template <bool FULL>
__device__ __forceinline__ float seg_causal(float* v, int len, float c) {
#pragma unroll
    for (int k = 0; k < kBandSeg; ++k) {
        if (FULL || k < len) {
            c = fmaf(kZ1, c, v[k]);
            v[k] = c;
        }
    }
    float e = 0.f;
#pragma unroll
    for (int k = kBandSeg - 1; k >= 0; --k)
        if (FULL || k < len) e = fmaf(kZ1, e, v[k]);
    return e;
}

// out points at sample len - 1 of the segment's output (stride ks)
template <bool FULL>
__device__ __forceinline__ void seg_anticausal(const float* v, int len, float c, float* out,
                                               int ks) {
    constexpr float gain = -6.0f * kZ1;
#pragma unroll
    for (int k = kBandSeg - 1; k >= 0; --k) {
        if (FULL || k < len) {
            c = fmaf(kZ1, c, v[k]);
            *out = gain * c;
            out -= ks;
        }
    }
}

// One periodic prefilter pass over `lines` lines of N samples: sample k of line l is
// in[l * ls + k * ks] (times the annular mask at (l, k) when MASK), its result goes to
// out[l * ls + k * ks] (out may be in); GLOBAL: in and out are global memory, else shared.  Each line is split into nsg segments of kBandSeg
// samples (the last one N - 32 (nsg - 1) long), one thread per segment with the segment in
// registers.  Lines go in rounds of LPR = 32 floor(NT / (32 nsg)), a warp holding one segment
// of 32 consecutive lines (so a warp's segments have one length).  Causal pass
// c+[k] = x[k] + z1 c+[k-1]: each thread forms its segment's end state from zero,
// E_g = sum_k z1^(L_g - 1 - k) x[k], and starts its recursion from E_{g-1} + z1^L_{g-1} E_{g-2}
// (periodic in g; the omitted terms are below z1^58 = 6e-34 of the state).  The anticausal pass
// c-[k] = c+[k] + z1 c-[k+1] does the same from the right, and the output is -6 z1 c-[k].
// carry holds 2 NT floats.  Ends with a barrier.
template <int NT, bool GLOBAL, bool MASK>
__device__ __forceinline__ void prefilter_lines(int lines, int N, int nsg, float zlast,
                                                float* carry, const float* in, float* out,
                                                int ls, int ks) {
    constexpr float zseg = rot::z1_pow<kBandSeg>();
    const int lpr = 32 * (NT / (32 * nsg));
    const int t = threadIdx.x;
    const int lw = t % lpr, g = t / lpr;
    const bool has_seg = g < nsg;
    const int k0 = g * kBandSeg;
    const int len = has_seg ? min(kBandSeg, N - k0) : 0;
    const bool full = len == kBandSeg;               // the same for a whole warp
    float* carry_c = carry;              // [nsg][lpr] causal end states
    float* carry_a = carry + NT;         // [nsg][lpr] anticausal start states
    const int g1 = g == 0 ? nsg - 1 : g - 1, g2 = g1 == 0 ? nsg - 1 : g1 - 1;
    const int h1 = g == nsg - 1 ? 0 : g + 1, h2 = h1 == nsg - 1 ? 0 : h1 + 1;
    const float zg1 = g1 == nsg - 1 ? zlast : zseg;
    const float zh1 = h1 == nsg - 1 ? zlast : zseg;
    for (int l0 = 0; l0 < lines; l0 += lpr) {
        const int l = l0 + lw;
        const bool active = has_seg && l < lines;
        const int off = l * ls + k0 * ks;
        float v[kBandSeg];
        if (active)
            carry_c[g * lpr + lw] =
                    full ? seg_causal_end<true, GLOBAL, MASK>(v, len, in + off, ks, N, l, k0)
                         : seg_causal_end<false, GLOBAL, MASK>(v, len, in + off, ks, N, l, k0);
        __syncthreads();
        if (active) {
            const float c = fmaf(zg1, carry_c[g2 * lpr + lw], carry_c[g1 * lpr + lw]);
            carry_a[g * lpr + lw] = full ? seg_causal<true>(v, len, c)
                                         : seg_causal<false>(v, len, c);
        }
        __syncthreads();
        if (active) {
            const float c = fmaf(zh1, carry_a[h2 * lpr + lw], carry_a[h1 * lpr + lw]);
            float* o = out + off + (len - 1) * ks;
            if (full)
                seg_anticausal<true>(v, len, c, o, ks);
            else
                seg_anticausal<false>(v, len, c, o, ks);
        }
        __syncthreads();
    }
}

// One output sample from the band: layout coordinates (U, V) in 32.32 fixed point with the
// window's -1 folded in, band row rho = the window's first layout row - b0, iv its first
// layout column.
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

// Two output samples a, b from the band with paired FP32 instructions (as sample_fixed2 does
// for the whole-image kernel): layout coordinates (U, V) in 32.32 fixed point with the window's
// -1 folded in (see sample_band).
__device__ __forceinline__ float2 sample_band2(const float* s, int P, int rho_a, int iv_a,
                                               int64_t Ua, int64_t Va, int rho_b, int iv_b,
                                               int64_t Ub, int64_t Vb) {
    const float2 k32 = make_float2(2.3283064365386963e-10f, 2.3283064365386963e-10f);
    const float2 tu = __fmul2_rn(make_float2((float)(uint32_t)(Ua & 0xffffffffll),
                                             (float)(uint32_t)(Ub & 0xffffffffll)), k32);
    const float2 tv = __fmul2_rn(make_float2((float)(uint32_t)(Va & 0xffffffffll),
                                             (float)(uint32_t)(Vb & 0xffffffffll)), k32);
    float2 wu[4], wv[4];
    rot::bspline_w2(tu, wu);
    rot::bspline_w2(tv, wv);
    const float* a = s + rho_a * P + iv_a;
    const float* b = s + rho_b * P + iv_b;
    float2 acc = make_float2(0.f, 0.f);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        float2 v = __fmul2_rn(wv[0], make_float2(a[i * P], b[i * P]));
        v = __ffma2_rn(wv[1], make_float2(a[i * P + 1], b[i * P + 1]), v);
        v = __ffma2_rn(wv[2], make_float2(a[i * P + 2], b[i * P + 2]), v);
        v = __ffma2_rn(wv[3], make_float2(a[i * P + 3], b[i * P + 3]), v);
        acc = __ffma2_rn(wu[i], v, acc);
    }
    return acc;
}

// One rotation: the layout-column prefilter from `in` to A, then the bands.  TRANS: `in` is
// transposed (layout row u = reference column), masked with the annular mask on load.
template <int NT, bool TRANS, bool PAIRED>
__device__ __forceinline__ void rotate_banded(const float* in, float* A, float* out, float* s,
                                              float* carry, const RotConst* Qp, int N, int P1,
                                              int Pm1, int H0, int nb, int nsg, float zlast) {
    // 1. along layout columns: line = column v, sample k = row u
    // (TRANS: layout (u, v) is reference (v, u), masked by mask_ref(v, u))
    prefilter_lines<NT, true, TRANS>(N, N, nsg, zlast, carry, in, A, 1, N);
    // The band's row stride: a warp's lanes sample along an output row, a layout step of
    // (rc, rs) (TRANS) or (rs, rc) per lane; tap (rho, iv) sits in bank (rho P + iv) mod 32, so
    // P = 1 mod 32 keeps the bank index monotone across the lanes when the two components have
    // one sign and P = -1 mod 32 when they have opposite signs (about two wavefronts per tap
    // instruction either way, as in the whole-image kernels).  Qp is in shared memory, written
    // before the column pass's barriers.
    const int P = (Qp->rc > 0) == (Qp->rs > 0) ? P1 : Pm1;
    constexpr int64_t kOne = 1ll << 32;
    const int R = NT / N;
    const int c = threadIdx.x % N, r0 = threadIdx.x / N;
#pragma unroll 1
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
        // +-1 mod 32, so a warp's 32 accesses fall in 32 banks)
        prefilter_lines<NT, false, false>(rows, N, nsg, zlast, carry, s, s, P, 1);
        for (int p = threadIdx.x; p < rows * 3; p += NT) {
            const int rho = p / 3, j = p - rho * 3;
            s[rho * P + N + j] = s[rho * P + j];
        }
        __syncthreads();
        // 2c. every output whose window starts in the band.  Thread (c, r0) owns rows
        // r0 + j R, j < J; along them the window's first layout row U_j = U_0 + j dU is linear,
        // so the rows in the band (its rows b0 .. b0 + h - 1, met as U in [b0, b0 + h) + k N,
        // k = -1, 0, 1, since U stays within (-N, 2N)) are up to three ranges of j, found from
        // U_0 and dU and widened by one step each way.  A warp walks the union of its lanes'
        // ranges in step (its samples then lie along output rows, as in the whole-image
        // kernels), two rows per iteration, and each sample checks its own row.
        {
            // the constants are read from shared memory after the band's barriers, so that
            // nothing of the sampling stays live in registers through the prefilter
            const RotConst Q = *Qp;
            const bool lane_ok = r0 < R;
            const int64_t X0 = Q.bx - kOne + (int64_t)r0 * Q.rc + (int64_t)c * Q.rs;
            const int64_t Y0 = Q.by - kOne - (int64_t)r0 * Q.rs + (int64_t)c * Q.rc;
            const int64_t dX = (int64_t)R * Q.rc, dY = -(int64_t)R * Q.rs;
            const int64_t U0 = TRANS ? Y0 : X0, dU = TRANS ? dY : dX;
            const int J = lane_ok ? (N - r0 + R - 1) / R : 0;
#pragma unroll 1
            for (int k = -1; k <= 1; ++k) {
                int j0 = 0, j1 = J;
                if (dU != 0) {
                    // in layout rows: U_0 / 2^32 and dU / 2^32 (float is exact enough here:
                    // the range is widened by a step each way)
                    const float u0 = (float)U0 * 2.3283064365386963e-10f;
                    const float inv = 4294967296.0f / (float)dU;
                    const float ea = ((float)(b0 + k * N) - u0) * inv;
                    const float eb = ((float)(b0 + h + k * N) - u0) * inv;
                    const float lo = fminf(fmaxf(fminf(ea, eb), -2.f), (float)J + 2.f);
                    const float hi = fminf(fmaxf(fmaxf(ea, eb), -2.f), (float)J + 2.f);
                    j0 = max(0, (int)floorf(lo) - 1);
                    j1 = min(J, (int)ceilf(hi) + 1);
                } else if (k != 0) {
                    j1 = 0;                        // a constant U: one pass (k = 0) over all rows
                }
                const bool some = j0 < j1;
                const int w0 = __reduce_min_sync(0xffffffffu, some ? j0 : 0x7fffffff);
                const int w1 = __reduce_max_sync(0xffffffffu, some ? j1 : 0);
                if (w0 >= w1) continue;            // warp-uniform
                int64_t X = X0 + (int64_t)w0 * dX, Y = Y0 + (int64_t)w0 * dY;
                if constexpr (!PAIRED) {
#pragma unroll 1
                    for (int j = w0; j < w1; ++j, X += dX, Y += dY) {
                        const int64_t U = TRANS ? Y : X, V = TRANS ? X : Y;
                        const int f = (int)(U >> 32);
                        const int rho = (dU == 0 ? wrap_n(f, N) : f - k * N) - b0;
                        if (j >= J || (unsigned)rho >= (unsigned)h) continue;
                        out[(int64_t)(r0 + j * R) * N + c] =
                                sample_band(s, P, rho, wrap_n((int)(V >> 32), N), U, V);
                    }
                    continue;
                }
#pragma unroll 1
                for (int j = w0; j < w1; j += 2, X += 2 * dX, Y += 2 * dY) {
                    const int64_t Ua = TRANS ? Y : X, Va = TRANS ? X : Y;
                    const int64_t Ub = Ua + dU, Vb = Va + (TRANS ? dX : dY);
                    const int fa = (int)(Ua >> 32), fb = (int)(Ub >> 32);
                    int ra = (dU == 0 ? wrap_n(fa, N) : fa - k * N) - b0;
                    int rb = (dU == 0 ? wrap_n(fb, N) : fb - k * N) - b0;
                    const bool in_a = j < J && (unsigned)ra < (unsigned)h;
                    const bool in_b = j + 1 < J && (unsigned)rb < (unsigned)h;
                    if (!(in_a || in_b)) continue;
                    ra = in_a ? ra : 0;            // a valid address for the unused half
                    rb = in_b ? rb : 0;
                    const float2 v = sample_band2(s, P, ra, wrap_n((int)(Va >> 32), N), Ua, Va,
                                                  rb, wrap_n((int)(Vb >> 32), N), Ub, Vb);
                    if (in_a) out[(int64_t)(r0 + j * R) * N + c] = v.x;
                    if (in_b) out[(int64_t)(r0 + (j + 1) * R) * N + c] = v.y;
                }
            }
        }
        __syncthreads();
    }
}

// xbuf: the low-passed image (storage orientation), then the first rotation's output; A: the
// image's spectrum slot (>= N^2 floats, free at this point) as coefficient scratch.
template <int NT, int MINB, bool PAIRED>
__global__ void __launch_bounds__(NT, MINB) rotate_band_kernel(
        float* xbuf, float2* spec, int64_t Kc, float* img_out, const RotConst* __restrict__ rotc,
        int N, int P1, int Pm1, int H0, int nb, int nsg, float zlast) {
    extern __shared__ float sm[];
    float* carry = sm;                   // 2 NT floats
    float* s = sm + 2 * NT;              // (H0 + 3) x max(P1, Pm1) band
    const int64_t img = blockIdx.x;
    const int64_t NN = (int64_t)N * N;
    float* B = xbuf + img * NN;
    float* A = reinterpret_cast<float*>(spec + img * Kc);
    __shared__ RotConst rq[2];
    if (threadIdx.x < 2) rq[threadIdx.x] = rotc[2 * img + threadIdx.x];
    // rq is read after the first column pass's barriers; B is read by that pass before any
    // band writes it
    rotate_banded<NT, true, PAIRED>(B, A, B, s, carry, rq, N, P1, Pm1, H0, nb, nsg, zlast);
    rotate_banded<NT, false, PAIRED>(B, A, img_out + img * NN, s, carry, rq + 1, N, P1, Pm1, H0,
                                     nb, nsg, zlast);
}

}  // namespace

namespace kern {

bool rotate_band_supported(int N) { return N >= 64 && N <= kMaxBandN; }

int rotate_band(const mem_plan& P, float* xbuf, float2* spec, float* img_out, const void* rotc,
                cudaStream_t s) {
    if (P.n_images == 0) return MEM_OK;
    const int N = P.N;
    if (!rotate_band_supported(N) || P.Kc * 2 < (int64_t)N * N) return MEM_ERR_UNSUPPORTED;
    // row strides >= N + 3 (the 3-column halo), one = 1 mod 32 and one = -1 mod 32 (the
    // rotation picks one by its angle, see rotate_banded)
    const int P1 = ((N + 3 + 30) / 32) * 32 + 1;
    const int Pm1 = ((N + 3 + 32) / 32) * 32 - 1;
    const int Pst = std::max(P1, Pm1);
    // variant 0: one sample per step, 512 threads, two CTAs per SM; 1: two samples per step
    // (paired FP32), 512 threads, two CTAs per SM; 2: two samples per step, 512 threads, one CTA
    // per SM with the larger register file and bands up to 200 KB; 3: two samples per step,
    // 1024 threads, one CTA per SM, bands up to 200 KB.  Bands: the fewest within the
    // shared-memory budget (MEM_ROT_BANDS asks for more).
    const int variant = P.rot_band_variant;
    const int NT = variant == 3 ? 1024 : kBandThreads;
    const size_t budget = (variant >= 2 ? 200 * 1024 : 100 * 1024) - 2 * NT * sizeof(float);
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
    auto kfn = variant == 3   ? rotate_band_kernel<1024, 1, true>
               : variant == 2 ? rotate_band_kernel<kBandThreads, 1, true>
               : variant == 1 ? rotate_band_kernel<kBandThreads, 2, true>
                              : rotate_band_kernel<kBandThreads, 2, false>;
    MEM_CUDA_TRY(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
    kfn<<<(unsigned)P.n_images, NT, smem, s>>>(
            xbuf, spec, P.Kc, img_out, static_cast<const RotConst*>(rotc), N, P1, Pm1, H0, nb,
            nsg, zlast);
    MEM_LAUNCH_CHECK();
    return MEM_OK;
}

}  // namespace kern
}  // namespace mem
