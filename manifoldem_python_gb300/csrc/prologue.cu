// Image-side kernels of the distance stage (everything before the D contraction).
//
// Reference: modules/getDistanceCTF_local_Conj9combinedS2.py:216-400 and the helpers it calls
// (rotatefill.py, annularMask.py, ctemh_cryoFrank.py, get_wiener1 :422-430).
//
// Data layout in HBM (per call):
//   xbuf   [n_images][N][N] float   raw image (storage orientation), later scratch
//   spec   [n_images][N][N/2+1] float2   half-plane spectra (cuFFT R2C layout)
//   feats  [n_rows][Kf]  float (FP32 form) or two bf16 matrices hi/lo (split form):
//          column blocks U' | V' | r' | s' (see features_kernel)
#include <cuda_bf16.h>
#include <algorithm>
#include <cmath>

#include "mem_internal.cuh"
#include "rotate_fixed.cuh"

namespace mem {
namespace {

using namespace rot;

constexpr int kInitTaps = 18;                      // |z1|^18 = 5e-11


// Two Kahan-compensated float sums in paired FP32 instructions (fadd.rn.f32x2 / fma.rn.f32x2),
// the compensation kept negated, e = -c: y = x + e, t = s + y, e = (s - t) + y, s = t -- the
// same roundings as KSum below, so the sums are bit-identical to two KSum.
struct KSum2 {
    float2 s = make_float2(0.f, 0.f), e = make_float2(0.f, 0.f);
    __device__ __forceinline__ void add(float2 x) {
        const float2 y = __fadd2_rn(x, e);
        const float2 t = __fadd2_rn(s, y);
        e = __fadd2_rn(__ffma2_rn(t, make_float2(-1.f, -1.f), s), y);
        s = t;
    }
    __device__ __forceinline__ float2 value() const { return __fadd2_rn(s, e); }
};

// Kahan-compensated float accumulator
struct KSum {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x) {
        const float y = x - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ float value() const { return s - c; }
};

// background mean and 1/std of an image of NN pixels from per-thread partial sums a (values)
// and b (squares), red[2 NT / 32]: warp sums in FP64, then one thread adds the warp sums and
// forms the mean and 1/std (FP64 arithmetic is slow on this part; the other threads take the
// results from shared memory instead of repeating it)
template <int NT>
__device__ __forceinline__ void block_stats(double a, double b, double* red, int NN,
                                            float* mean, float* inv) {
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) {
        red[w] = a;
        red[NT / 32 + w] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0, t2 = 0.0;
#pragma unroll
        for (int i = 0; i < NT / 32; ++i) t += red[i];
#pragma unroll
        for (int i = 0; i < NT / 32; ++i) t2 += red[NT / 32 + i];
        const double m = t / NN;
        red[0] = m;
        red[1] = 1.0 / sqrt(fmax(t2 / NN - m * m, 0.0));
    }
    __syncthreads();
    *mean = (float)red[0];
    *inv = (float)red[1];
}

template <int NT>
__device__ __forceinline__ double block_sum_double(double v, double* red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x < 32) {
        t = (threadIdx.x < NT / 32) ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (threadIdx.x == 0) red[0] = t;
    }
    __syncthreads();
    return red[0];
}

// ------------------------------------------------------------------------------------------
// 1. gather + conjugate flip + background normalisation (reference :245-283)
//
// The reference image is I[r][c] = stack[idx][c][r] (memmap(...).T), flipped up-down for
// conjugate views.  The kernel writes it transposed ("storage orientation": out[a][b] = I[b][a])
// so that reads and writes are both contiguous rows of the stack.  The low-pass filter is
// symmetric in (kx, ky), so the transpose commutes with it; the rotation kernel undoes it.
// ------------------------------------------------------------------------------------------
template <int NT>
__device__ __forceinline__ void gather_normalize_one(
        int64_t img, const float* __restrict__ stack, int64_t num_stack,
        const int64_t* __restrict__ sidx, const uint8_t* __restrict__ flip,
        float* __restrict__ xbuf, int N, uint32_t* __restrict__ status, double* red) {
    const int64_t s = sidx[img];
    const int NN = N * N;
    float* dst = xbuf + img * (int64_t)NN;
    if (s < 0 || s >= num_stack) {                  // out-of-range index: flag and emit NaN
        if (threadIdx.x == 0) atomicOr(status, 2u);
        for (int p = threadIdx.x; p < NN; p += NT) dst[p] = __int_as_float(0x7fc00000);
        return;
    }
    const bool f = flip[img] != 0;
    const float* src = stack + s * (int64_t)NN;
    KSum sum, sq;
    for (int p = threadIdx.x; p < NN; p += NT) {
        const int a = p / N, b = p - a * N;
        const float v = src[a * N + (f ? N - 1 - b : b)];
        const float bg = v * (1.0f - mask_ref(b, a, N));   // reference pixel (r=b, c=a)
        sum.add(bg);
        sq.add(bg * bg);
    }
    static_assert(NT <= 512, "red[32] holds two sets of warp sums");
    float fmean, inv;
    block_stats<NT>((double)sum.value(), (double)sq.value(), red, NN, &fmean, &inv);
    for (int p = threadIdx.x; p < NN; p += NT) {
        const int a = p / N, b = p - a * N;
        dst[p] = (src[a * N + (f ? N - 1 - b : b)] - fmean) * inv;
    }
}

// one CTA per image, or a smaller grid looping over the images
template <int NT>
__global__ void __launch_bounds__(NT) gather_normalize_kernel(
        const float* __restrict__ stack, int64_t num_stack, const int64_t* __restrict__ sidx,
        const uint8_t* __restrict__ flip, float* __restrict__ xbuf, int N,
        uint32_t* __restrict__ status, int64_t n_images) {
    __shared__ double red[32];
    for (int64_t img = blockIdx.x; img < n_images; img += gridDim.x) {
        __syncthreads();
        gather_normalize_one<NT>(img, stack, num_stack, sidx, flip, xbuf, N, status, red);
    }
}

// raw copy of every entry's stack image into slot i of out (a stack in host memory read over
// the host link by a few light CTAs; the arithmetic then runs on the copies)
__global__ void __launch_bounds__(1024) gather_copy_kernel(
        const float* __restrict__ stack, int64_t num_stack, const int64_t* __restrict__ sidx,
        int64_t n_images, int NN, float* __restrict__ out, uint32_t* __restrict__ status) {
    // two images per step (CTA images img and img + gridDim.x), their 16-byte loads issued
    // before the stores, so that a small grid keeps enough reads in flight on the host link
    const int64_t step = 2 * (int64_t)gridDim.x;
    for (int64_t img = blockIdx.x; img < n_images; img += step) {
        const int64_t img2 = img + gridDim.x;
        const int n_img = img2 < n_images ? 2 : 1;
        const float* src[2];
        float* dst[2];
        bool ok[2];
        for (int q = 0; q < 2; ++q) {
            const int64_t im = q == 0 ? img : img2;
            const int64_t s = q < n_img ? sidx[im] : -1;
            ok[q] = q < n_img && s >= 0 && s < num_stack;
            src[q] = stack + (ok[q] ? s : 0) * (int64_t)NN;
            dst[q] = out + im * (int64_t)NN;
            if (q < n_img && !ok[q]) {
                if (threadIdx.x == 0) atomicOr(status, 2u);
                for (int p = threadIdx.x; p < NN; p += blockDim.x)
                    dst[q][p] = __int_as_float(0x7fc00000);
            }
        }
        if ((NN & 3) == 0) {
            const int NQ = NN / 4;
            const float4* s0 = reinterpret_cast<const float4*>(src[0]);
            const float4* s1 = reinterpret_cast<const float4*>(src[1]);
            float4* d0 = reinterpret_cast<float4*>(dst[0]);
            float4* d1 = reinterpret_cast<float4*>(dst[1]);
            for (int p0 = threadIdx.x; p0 < NQ; p0 += 4 * blockDim.x) {
                float4 v[2][4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int p = p0 + u * blockDim.x;
                    if (p < NQ) {
                        if (ok[0]) v[0][u] = s0[p];
                        if (ok[1]) v[1][u] = s1[p];
                    }
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int p = p0 + u * blockDim.x;
                    if (p < NQ) {
                        if (ok[0]) d0[p] = v[0][u];
                        if (ok[1]) d1[p] = v[1][u];
                    }
                }
            }
        } else {
            for (int q = 0; q < 2; ++q) {
                if (!ok[q]) continue;
#pragma unroll 8
                for (int p = threadIdx.x; p < NN; p += blockDim.x) dst[q][p] = src[q][p];
            }
        }
    }
}

// float4 variant for N % 4 == 0: one 16-byte load / store per 4 pixels of a stack row; a
// conjugate flip reverses the four lanes (the row reversal maps aligned quads to aligned quads)
template <int NT>
__device__ __forceinline__ void gather_normalize_v4_one(
        int64_t img, const float* __restrict__ stack, int64_t num_stack,
        const int64_t* __restrict__ sidx, const uint8_t* __restrict__ flip,
        float* __restrict__ xbuf, int N, uint32_t* __restrict__ status, double* red) {
    const int64_t s = sidx[img];
    const int NN = N * N, NQ = NN / 4;
    float4* dst = reinterpret_cast<float4*>(xbuf + img * (int64_t)NN);
    if (s < 0 || s >= num_stack) {
        if (threadIdx.x == 0) atomicOr(status, 2u);
        const float nan = __int_as_float(0x7fc00000);
        for (int p = threadIdx.x; p < NQ; p += NT) dst[p] = make_float4(nan, nan, nan, nan);
        return;
    }
    const bool f = flip[img] != 0;
    const float4* src = reinterpret_cast<const float4*>(stack + s * (int64_t)NN);
    auto load = [&](int p, int& a, int& b) -> float4 {
        const int e = 4 * p;
        a = e / N;
        b = e - a * N;
        float4 v = src[(a * N + (f ? N - 4 - b : b)) >> 2];
        if (f) v = make_float4(v.w, v.z, v.y, v.x);
        return v;
    };
    KSum sum, sq;
    for (int p = threadIdx.x; p < NQ; p += NT) {
        int a, b;
        const float4 v = load(p, a, b);
        const float vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float bg = vv[j] * (1.0f - mask_ref(b + j, a, N));   // reference pixel (b+j, a)
            sum.add(bg);
            sq.add(bg * bg);
        }
    }
    static_assert(NT <= 512, "red[32] holds two sets of warp sums");
    float fmean, inv;
    block_stats<NT>((double)sum.value(), (double)sq.value(), red, NN, &fmean, &inv);
    for (int p = threadIdx.x; p < NQ; p += NT) {
        int a, b;
        const float4 v = load(p, a, b);
        dst[p] = make_float4((v.x - fmean) * inv, (v.y - fmean) * inv, (v.z - fmean) * inv,
                             (v.w - fmean) * inv);
    }
}

// one CTA per image, or a smaller grid looping over the images
template <int NT>
__global__ void __launch_bounds__(NT) gather_normalize_v4_kernel(
        const float* __restrict__ stack, int64_t num_stack, const int64_t* __restrict__ sidx,
        const uint8_t* __restrict__ flip, float* __restrict__ xbuf, int N,
        uint32_t* __restrict__ status, int64_t n_images) {
    __shared__ double red[32];
    for (int64_t img = blockIdx.x; img < n_images; img += gridDim.x) {
        __syncthreads();
        gather_normalize_v4_one<NT>(img, stack, num_stack, sidx, flip, xbuf, N, status, red);
    }
}

// ------------------------------------------------------------------------------------------
// 2. low-pass filter table G(k)/N^2 and its application (reference :139-167, :286-293)
// ------------------------------------------------------------------------------------------
__global__ void lowpass_table_kernel(float* __restrict__ g, int N, int Nh, int type, double Qc,
                                     double order) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= N * Nh) return;
    const int ka = k / Nh, kb = k - ka * Nh;
    const int fa = min(ka, N - ka), fb = kb;
    const double Q = sqrt((double)(fa * fa + fb * fb)) / (N / 2.0);
    double G;
    if (type == MEM_FILTER_GAUSS)
        G = exp(-(log(2.0) / 2.0) * (Q / Qc) * (Q / Qc));
    else
        G = sqrt(1.0 / (1.0 + pow(Q / Qc, 2.0 * order)));
    g[k] = (float)(G / ((double)N * N));
}

__global__ void lowpass_apply_kernel(float2* __restrict__ spec, const float* __restrict__ g,
                                     int64_t total, int KcN) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const float gv = g[e % KcN];
        float2 v = spec[e];
        v.x *= gv;
        v.y *= gv;
        spec[e] = v;
    }
}

// ------------------------------------------------------------------------------------------
// 3. mask + two periodic cubic B-spline rotations (reference :326-330, rotatefill.py:21-25)
//
// rotatefill tiles the image 3x3 and calls scipy.ndimage.rotate(order=3); that is a periodic
// cubic B-spline rotation about ((N-1)/2, (N-1)/2):
//   out[r][c] = sum_{i,j} coef[x_i][y_j] B3(x - x_i) B3(y - y_j),
//   x = cos t (r-c0) + sin t (c-c0) + c0,  y = -sin t (r-c0) + cos t (c-c0) + c0.
// coef is the periodic prefilter of the image: the causal/anticausal recursion with pole
// z1 = sqrt(3) - 2, each row (then column) split into segments.  The runtime-size kernels start
// each segment from the truncated geometric sum over the previous kInitTaps samples (exact to
// |z1|^18); the compile-time kernels hold the segments in registers and start them from their
// neighbours' end states (prefilter_fixed).  Sample coordinates are computed in 64-bit fixed
// point (32 fractional bits) from constants made once per image (rot_const_kernel).
// ------------------------------------------------------------------------------------------
// The two rotations of every image: rotatefill by -(180/pi) Psi_i degrees (back to radians),
// then by the PD's -psi_p (its cosine and sine are in the PD table).  Computed once per image so
// that the rotation kernels read them instead of one thread per CTA evaluating FP64
// trigonometry while the CTA waits (FP64 is slow on this part).
__global__ void rot_const_kernel(const double* __restrict__ psi_rad, const PdDev* __restrict__ pds,
                                 const int32_t* __restrict__ img_pd, RotConst* __restrict__ out,
                                 int64_t n, int N) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double ang = -(180.0 / 3.141592653589793) * psi_rad[i];
    const double t = ang * (3.141592653589793 / 180.0);
    out[2 * i] = make_rot(cos(t), sin(t), N);
    const PdDev& pd = pds[img_pd[i]];
    out[2 * i + 1] = make_rot(pd.rot2_cos, pd.rot2_sin, N);
}

// one axis of the periodic prefilter over an N x N image in smem (row stride P).
// axis 0: filter along each row (elements s[r*P + k]); axis 1: along each column.
template <int NT>
__device__ void prefilter_axis(float* s, int N, int P, int axis, int nseg, float inv1mzN,
                               bool exact_init) {
    const int seg_len = (N + nseg - 1) / nseg;
    const int lines = N * nseg;
    const int stride_k = axis == 0 ? 1 : P;
    const int stride_l = axis == 0 ? P : 1;
    const int taps = exact_init ? N : kInitTaps;
    float init = 0.f;
    int line = 0, k0 = 0, k1 = -1;
    const int t = threadIdx.x;
    const bool active = t < lines;
    if (active) {
        line = t % N;
        const int g = t / N;
        k0 = g * seg_len;
        k1 = min(N, k0 + seg_len) - 1;
    }
    float* base = s + line * stride_l;
    // causal start value c+[k0] = sum_j z1^j s[k0 - j]
    if (active && k0 <= k1) {
        float acc = 0.f, zp = 1.f;
        for (int j = 0; j < taps; ++j) {      // taps <= N: one wrap at most
            int idx = k0 - j;
            idx += (idx < 0) ? N : 0;
            acc += zp * base[idx * stride_k];
            zp *= kZ1;
        }
        init = exact_init ? acc * inv1mzN : acc;
    }
    __syncthreads();
    if (active && k0 <= k1) {
        float prev = init;
        base[k0 * stride_k] = prev;
        for (int k = k0 + 1; k <= k1; ++k) {
            prev = base[k * stride_k] + kZ1 * prev;
            base[k * stride_k] = prev;
        }
    }
    __syncthreads();
    // anticausal start value c-[k1] = sum_j z1^j c+[k1 + j]
    if (active && k0 <= k1) {
        float acc = 0.f, zp = 1.f;
        for (int j = 0; j < taps; ++j) {
            int idx = k1 + j;
            idx -= (idx >= N) ? N : 0;
            acc += zp * base[idx * stride_k];
            zp *= kZ1;
        }
        init = exact_init ? acc * inv1mzN : acc;
    }
    __syncthreads();
    if (active && k0 <= k1) {
        const float gain = -6.0f * kZ1;
        float prev = init;
        base[k1 * stride_k] = gain * prev;
        for (int k = k1 - 1; k >= k0; --k) {
            prev = base[k * stride_k] + kZ1 * prev;
            base[k * stride_k] = gain * prev;
        }
    }
    __syncthreads();
}

// wrapped index of i in [-N, 2N)
__device__ __forceinline__ int wrapN(int i, int N) {
    i += (i < 0) ? N : 0;
    return i - ((i >= N) ? N : 0);
}

// one output sample at fixed-point coordinates (X, Y) (32 fractional bits)
__device__ __forceinline__ float sample_at(const float* s, int N, int P, int64_t X, int64_t Y) {
    const int ix = (int)(X >> 32), iy = (int)(Y >> 32);
    const float tx = (float)(uint32_t)(X & 0xffffffffll) * 2.3283064365386963e-10f;
    const float ty = (float)(uint32_t)(Y & 0xffffffffll) * 2.3283064365386963e-10f;
    float wx[4], wy[4];
    bspline_w(tx, wx);
    bspline_w(ty, wy);
    const float* base = s + wrapN(ix - 1, N) * P + wrapN(iy - 1, N);
    float acc = 0.f;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float* row = base + i * P;
        const float v = wy[0] * row[0] + wy[1] * row[1] + wy[2] * row[2] + wy[3] * row[3];
        acc = fmaf(wx[i], v, acc);
    }
    return acc;
}

// Thread t owns column c = t % N and rows r = t / N + k R (R = NT / N rows per pass), so its
// sample coordinates advance by a constant fixed-point step.  A warp's lanes sample along an
// output row, a step of (rs, rc) in (x, y); tap (ix, iy) sits in bank (ix P + iy) mod 32, so each
// rotation lays its coefficient image out with row stride P1 = 1 mod 32 when rc and rs have one
// sign and Pm1 = -1 mod 32 otherwise (a monotone bank index across the lanes: about two
// wavefronts per tap instruction); P1 = Pm1 = an odd stride where those do not fit.
template <int NT, int MAXV>
__global__ void __launch_bounds__(NT) rotate_kernel(
        float* __restrict__ xbuf, float* __restrict__ img_out, const RotConst* __restrict__ rotc,
        int N, int P1, int Pm1, int nseg, float inv1mzN, int exact_init) {
    extern __shared__ float s[];
    const int64_t img = blockIdx.x;
    const RotConst q0 = rotc[2 * img], q1 = rotc[2 * img + 1];
    const int Pa = (q0.rc > 0) == (q0.rs > 0) ? P1 : Pm1;
    const int Pb = (q1.rc > 0) == (q1.rs > 0) ? P1 : Pm1;
    const int NN = N * N;
    float* xi = xbuf + img * (int64_t)NN;
    const int R = NT / N;                       // rows per pass
    const int c = threadIdx.x % N;
    const int r0 = threadIdx.x / N;
    const bool active = r0 < R;
    // load (storage orientation) into smem in reference orientation, times the mask
    for (int p = threadIdx.x; p < NN; p += NT) {
        const int a = p / N, b = p - a * N;
        s[b * Pa + a] = xi[p] * mask_ref(b, a, N);
    }
    __syncthreads();
    prefilter_axis<NT>(s, N, Pa, 0, nseg, inv1mzN, exact_init != 0);
    prefilter_axis<NT>(s, N, Pa, 1, nseg, inv1mzN, exact_init != 0);
    fill_halo<NT>(s, N, Pa);
    float keep[MAXV > 0 ? MAXV : 1];
    {
        const RotConst& Q = q0;
        int64_t X = Q.bx + (int64_t)r0 * Q.rc + (int64_t)c * Q.rs;
        int64_t Y = Q.by - (int64_t)r0 * Q.rs + (int64_t)c * Q.rc;
        const int64_t dX = (int64_t)R * Q.rc, dY = -(int64_t)R * Q.rs;
        if (MAXV > 0) {
#pragma unroll
            for (int k = 0; k < MAXV; ++k) {
                const int r = r0 + k * R;
                if (active && r < N) keep[k] = sample_at(s, N, Pa, X, Y);
                X += dX;
                Y += dY;
            }
        } else if (active) {
            for (int r = r0; r < N; r += R, X += dX, Y += dY)
                xi[r * N + c] = sample_at(s, N, Pa, X, Y);
        }
    }
    __syncthreads();
    if (MAXV > 0) {
#pragma unroll
        for (int k = 0; k < MAXV; ++k) {
            const int r = r0 + k * R;
            if (active && r < N) s[r * Pb + c] = keep[k];
        }
    } else {
        for (int p = threadIdx.x; p < NN; p += NT) {
            const int r = p / N, cc = p - r * N;
            s[r * Pb + cc] = xi[p];
        }
    }
    __syncthreads();
    prefilter_axis<NT>(s, N, Pb, 0, nseg, inv1mzN, exact_init != 0);
    prefilter_axis<NT>(s, N, Pb, 1, nseg, inv1mzN, exact_init != 0);
    fill_halo<NT>(s, N, Pb);
    if (!active) return;
    const RotConst& Q = q1;
    int64_t X = Q.bx + (int64_t)r0 * Q.rc + (int64_t)c * Q.rs;
    int64_t Y = Q.by - (int64_t)r0 * Q.rs + (int64_t)c * Q.rc;
    const int64_t dX = (int64_t)R * Q.rc, dY = -(int64_t)R * Q.rs;
    float* out = img_out + img * (int64_t)NN;
    for (int r = r0; r < N; r += R, X += dX, Y += dY) out[r * N + c] = sample_at(s, N, Pb, X, Y);
}

// Compile-time box size (power-of-two N, 512 threads): the same computation as rotate_kernel
// with every loop bound, row stride and tap offset a constant, the tap indices wrapped by a
// mask, the -1 of the 4-tap window folded into the fixed-point origin and the prefilter
// segments held in registers (prefilter_fixed).
template <int NT, int N>
__global__ void __launch_bounds__(NT, 2) rotate_fixed_kernel(
        float* __restrict__ xbuf, float* __restrict__ img_out, const RotConst* __restrict__ rotc) {
    constexpr int NN = N * N;
    extern __shared__ float s[];
    __shared__ RotConst rot[2];
    __shared__ float carry[2 * rot_nseg<NT, N>() * N];
    const int64_t img = blockIdx.x;
    if (threadIdx.x < 2) rot[threadIdx.x] = rotc[2 * img + threadIdx.x];
    // rot[] is read after the first prefilter's barriers
    rotate_image<NT, N, false>(xbuf + img * (int64_t)NN, img_out + img * (int64_t)NN, s, carry,
                               rot);
}

// Boxes too large for the shared-memory kernel (N > 236): the same two rotations with the spline
// coefficients in global memory (the image's own workspace slots, L1/L2-resident while the CTA
// works on them).  A = the image's spectrum slot (free at this point, >= N*N floats), B = its
// xbuf slot.  Row stride N, no halo: every tap index is wrapped.
__device__ __forceinline__ float sample_wrap(const float* s, int N, int64_t X, int64_t Y) {
    const int ix = (int)(X >> 32), iy = (int)(Y >> 32);
    const float tx = (float)(uint32_t)(X & 0xffffffffll) * 2.3283064365386963e-10f;
    const float ty = (float)(uint32_t)(Y & 0xffffffffll) * 2.3283064365386963e-10f;
    float wx[4], wy[4];
    bspline_w(tx, wx);
    bspline_w(ty, wy);
    int cols[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) cols[j] = wrapN(iy - 1 + j, N);
    float acc = 0.f;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float* row = s + wrapN(ix - 1 + i, N) * N;
        const float v = wy[0] * row[cols[0]] + wy[1] * row[cols[1]] + wy[2] * row[cols[2]] +
                        wy[3] * row[cols[3]];
        acc = fmaf(wx[i], v, acc);
    }
    return acc;
}

template <int NT>
__global__ void __launch_bounds__(NT) rotate_global_kernel(
        float* __restrict__ xbuf, float2* __restrict__ spec, int64_t Kc, float* __restrict__ img_out,
        const RotConst* __restrict__ rotc, int N, int nseg, float inv1mzN) {
    __shared__ RotConst rot[2];
    const int64_t img = blockIdx.x;
    const int NN = N * N;
    float* B = xbuf + img * (int64_t)NN;
    float* A = reinterpret_cast<float*>(spec + img * Kc);
    if (threadIdx.x < 2) rot[threadIdx.x] = rotc[2 * img + threadIdx.x];
    for (int p = threadIdx.x; p < NN; p += NT) {          // masked, back to reference orientation
        const int r = p / N, c = p - r * N;
        A[p] = B[c * N + r] * mask_ref(r, c, N);
    }
    __syncthreads();
    prefilter_axis<NT>(A, N, N, 0, nseg, inv1mzN, false);
    prefilter_axis<NT>(A, N, N, 1, nseg, inv1mzN, false);
    const int R = NT / N;
    const int c = threadIdx.x % N, r0 = threadIdx.x / N;
    const bool active = r0 < R;
    {
        const RotConst Q = rot[0];
        int64_t X = Q.bx + (int64_t)r0 * Q.rc + (int64_t)c * Q.rs;
        int64_t Y = Q.by - (int64_t)r0 * Q.rs + (int64_t)c * Q.rc;
        const int64_t dX = (int64_t)R * Q.rc, dY = -(int64_t)R * Q.rs;
        if (active)
            for (int r = r0; r < N; r += R, X += dX, Y += dY) B[r * N + c] = sample_wrap(A, N, X, Y);
    }
    __syncthreads();
    prefilter_axis<NT>(B, N, N, 0, nseg, inv1mzN, false);
    prefilter_axis<NT>(B, N, N, 1, nseg, inv1mzN, false);
    float* out = (img_out + img * (int64_t)NN == B) ? A : img_out + img * (int64_t)NN;
    {
        const RotConst Q = rot[1];
        int64_t X = Q.bx + (int64_t)r0 * Q.rc + (int64_t)c * Q.rs;
        int64_t Y = Q.by - (int64_t)r0 * Q.rs + (int64_t)c * Q.rc;
        const int64_t dX = (int64_t)R * Q.rc, dY = -(int64_t)R * Q.rs;
        if (active)
            for (int r = r0; r < N; r += R, X += dX, Y += dY) out[r * N + c] = sample_wrap(B, N, X, Y);
    }
    if (out == A) {
        __syncthreads();
        for (int p = threadIdx.x; p < NN; p += NT) B[p] = A[p];
    }
}

// ------------------------------------------------------------------------------------------
// CTF (ctemh_cryoFrank.py:24-44, called at :337-339) with an exact phase.
//   CTF = sin(wr) - A cos(wr) = sqrt(1 + A^2) sin(wr - atan A),   k^2 = m / (N pix)^2,
//   m = fa^2 + fb^2 the integer squared frequency index.  In cycles:
//   (wr - atan A) / 2pi = P m^2 - Q_i m - atan(A)/2pi,
//   P = Cs 1e7 lambda^3 / (4 (N pix)^4),  Q_i = lambda df_i / (2 (N pix)^2).
// The phase is reduced modulo one cycle in 64-bit fixed point, so its sign (and the phase
// flip sign(CTF)) is exact to ~1e-14 cycles and the value is float-accurate.
// ------------------------------------------------------------------------------------------
__global__ void qfix_kernel(const double* __restrict__ df, uint64_t* __restrict__ qfix,
                            int64_t n, double q_scale) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double q = q_scale * df[i];
    double fr = q - floor(q);
    double v = ldexp(fr, 64);
    qfix[i] = (v >= 18446744073709551615.0) ? 0ull : __double2ull_rn(v);
}

// sin(2 pi u / 2^64) of a phase u in 64-bit fixed-point cycles.  The top three bits give the
// octant o; the next 32 give y in [0, 1) (mirrored to 1 - y in odd octants), so that the value
// is +-sin(pi y / 4) (o mod 4 = 0, 3) or +-cos(pi y / 4) (o mod 4 = 1, 2), negative for o >= 4.
// Both are polynomials in y fitted here (weighted least squares on the relative error, each
// coefficient rounded to float in turn with the later ones refitted): max error 1.6 ulp (sin)
// and 0.9 ulp (cos) on [0, 1] in float arithmetic with fused multiply-adds; the float y adds at
// most pi/4 * 2^-24 = 4.7e-8 to the argument.
__device__ __forceinline__ float sin_cycles(uint64_t u) {
    const uint32_t o = (uint32_t)(u >> 61);
    uint32_t t = (uint32_t)(u >> 29);
    if (o & 1u) t = ~t;
    const float y = (float)t * 2.3283064365386963e-10f;     // t / 2^32
    const float y2 = y * y;
    float ps = fmaf(y2, -3.661072696559131e-05f, 0.0024910178035497665f);
    ps = fmaf(y2, ps, -0.08074583113193512f);
    ps = fmaf(y2, ps, 0.7853981852531433f);
    ps *= y;                                                // sin(pi y / 4)
    float pc = fmaf(y2, 3.4940505884151207e-06f, -0.0003258686629123986f);
    pc = fmaf(y2, pc, 0.015854284167289734f);
    pc = fmaf(y2, pc, -0.3084251284599304f);
    pc = fmaf(y2, pc, 1.0f);                                // cos(pi y / 4)
    const float v = ((o + 1u) & 2u) ? pc : ps;
    return (o & 4u) ? -v : v;
}

__device__ __forceinline__ float ctf_eval(int m, uint64_t qf, const CtfConst& cc, int* sgn) {
    const uint64_t mm = (uint32_t)m;                  // m >= 0: zero-extended
    const uint64_t ph = cc.p_fix * (mm * mm) - qf * mm - cc.d_fix;
    const int64_t sph = (int64_t)ph;
    *sgn = (sph > 0) - (sph < 0);
    float v = cc.amp * sin_cycles(ph);
    if (cc.env_c != 0.0f) v *= expf(-cc.env_c * (float)m);
    return v;
}

// ------------------------------------------------------------------------------------------
// 4. per-PD sums over images (partial, one item = up to kSumChunk images of one PD)
//    S0 = sum C^2, S1/S2 = sum C F, S3/S4 = sum sign(C) F, S5 = sum |F|^2
// ------------------------------------------------------------------------------------------
// WHICH: 1 = S0..S2 (the Wiener sums), 2 = S3..S5, 3 = all six
template <int WHICH>
__global__ void __launch_bounds__(256) pd_sums_kernel(
        const float2* __restrict__ spec, const uint64_t* __restrict__ qfix,
        const SumItem* __restrict__ items, float* __restrict__ partial, int N, int Nh, int64_t Kc,
        CtfConst cc) {
    const int64_t k = blockIdx.y * 256ll + threadIdx.x;
    const SumItem it = items[blockIdx.x];
    if (k < Kc) {
        const int ka = (int)(k / Nh), kb = (int)(k - (int64_t)ka * Nh);
        const int fa = min(ka, N - ka);
        const int m = fa * fa + kb * kb;
        KSum2 s05, s12, s34;        // (S0, S5), (S1, S2), (S3, S4)
#pragma unroll 4
        for (int64_t i = it.img_begin; i < it.img_end; ++i) {
            const float2 F = spec[i * Kc + k];
            int sg;
            float C = 0.f;
            if (WHICH & 1) {
                C = ctf_eval(m, qfix[i], cc, &sg);
                s12.add(__fmul2_rn(make_float2(C, C), F));
            } else {
                sg = ctf_sign(m, qfix[i], cc);
            }
            if (WHICH & 2) {
                const float g = (float)sg;
                s34.add(__fmul2_rn(make_float2(g, g), F));
            }
            s05.add(make_float2((WHICH & 1) ? C * C : 0.f,
                                (WHICH & 2) ? F.x * F.x + F.y * F.y : 0.f));
        }
        float* out = partial + (int64_t)blockIdx.x * 6 * Kc + k;
        const float2 v05 = s05.value(), v12 = s12.value(), v34 = s34.value();
        if (WHICH & 1) {
            out[0 * Kc] = v05.x;
            out[1 * Kc] = v12.x;
            out[2 * Kc] = v12.y;
        }
        if (WHICH & 2) {
            out[3 * Kc] = v34.x;
            out[4 * Kc] = v34.y;
            out[5 * Kc] = v05.y;
        }
    }
}

// 5. finalize: FP64 sum over the PD's items; centring vectors, average spectra, scale
__global__ void __launch_bounds__(256) pd_finalize_kernel(
        const float* __restrict__ partial, const SumItem* __restrict__ items,
        const int32_t* __restrict__ item_off, const PdDev* __restrict__ pds,
        const int32_t* __restrict__ ring_of, float* __restrict__ means,
        float2* __restrict__ avg_spec, uint32_t* __restrict__ pd_max,
        int N, int Nh, int64_t Kc, int64_t Kc_pad, int64_t mstride, int mode) {
    // mode bit 1: the Wiener average spectrum (from S0..S2); bit 2: centring vectors, scale and
    // the phase-flipped average spectrum.  With ring features (ring_of != null) the centring of
    // v is sw(k) mt(R) with the ring mean mt(R) = S0 / n of C^2 (the same sum for every member
    // of the ring: C depends on |k|^2 only), and mt(R) goes to the fifth block.
    const int64_t k = blockIdx.y * 256ll + threadIdx.x;
    const int pd = blockIdx.x;
    if (k >= Kc_pad) return;
    float* mu = means + pd * mstride;
    if (k >= Kc) {
        if (!(mode & 2)) return;
        mu[k] = mu[Kc_pad + k] = mu[2 * Kc_pad + k] = mu[3 * Kc_pad + k] = 0.f;
        return;
    }
    double S[6] = {0, 0, 0, 0, 0, 0};
    for (int it = item_off[pd]; it < item_off[pd + 1]; ++it) {
        const float* p = partial + (int64_t)it * 6 * Kc + k;
#pragma unroll
        for (int j = 0; j < 6; ++j) S[j] += (double)p[j * Kc];
    }
    // FP64 division is slow on this part: one reciprocal per factor, w in {1, 2} by constants
    const int n = pds[pd].n;
    const double NN = (double)N * N;
    const double inv_n = 1.0 / n, inv_nnn = 1.0 / (NN * n);
    float2* av = avg_spec + (int64_t)pd * 2 * Kc;
    if (mode & 1) {
        // Wiener average (reference :353-366): sum_i F_i C_i / -(sum C^2 + 1/5), / N^2, / n
        const double q = inv_nnn / -(S[0] + 0.2);
        av[k] = make_float2((float)(S[1] * q), (float)(S[2] * q));
    }
    if (!(mode & 2)) return;
    const int kb = (int)k % Nh;
    const bool w1 = kb == 0 || (N % 2 == 0 && kb == N / 2);
    const double sw = w1 ? 1.0 : 1.4142135623730951, s2w = w1 ? 1.4142135623730951 : 2.0;
    const float mu_u = (float)(sw * S[5] * inv_n);
    float mu_v = (float)(sw * S[0] * inv_n);
    if (ring_of) {
        const float mt = (float)(S[0] * inv_n);
        mu_v = (float)sw * mt;
        mu[4 * Kc_pad + ring_of[k]] = mt;
    }
    const float mu_r = (float)(s2w * S[1] * inv_n), mu_s = (float)(s2w * S[2] * inv_n);
    mu[k] = mu_u;
    mu[Kc_pad + k] = mu_v;
    mu[2 * Kc_pad + k] = mu_r;
    mu[3 * Kc_pad + k] = mu_s;
    const float mx = fmaxf(fmaxf(fabsf(mu_u), fabsf(mu_v)), fmaxf(fabsf(mu_r), fabsf(mu_s)));
    atomicMax(pd_max + pd, __float_as_uint(mx));
    // phase-flipped average (:346-348, :367): sum_i sign(C_i) F_i / N^2 / n
    av[Kc + k] = make_float2((float)(S[3] * inv_nnn), (float)(S[4] * inv_nnn));
}

// ------------------------------------------------------------------------------------------
// 6. features of one image (one CTA per image)
//   u = sqrt(w)|F|^2, v = sqrt(w) C^2, r = sqrt(2w) C Re F, s = sqrt(2w) C Im F, w the
//   half-plane weight; with x' = x - mean_PD(x):
//     D_ij = a_i + a_j + [u'_i.v'_j + v'_i.u'_j - r'_i.r'_j - s'_i.s'_j]
//     a_i  = sum_k (mu_u v_ik + mu_v u_ik - mu_u mu_v - mu_r r_ik + mu_r^2/2 - mu_s s_ik + mu_s^2/2)
//   (an exact rewrite of D_ij = sum_k |C_j F_i - C_i F_j|^2 for any centring vector mu).
//   Features are written scaled by the PD's power of two; a_i in FP64 unscaled.
//   With write_signed the spectrum is overwritten with sign(C) F / N^2 (input of a cuFFT
//   phase-flip C2R); the shared-memory inverse FFT applies sign(C) / N^2 itself.
// ------------------------------------------------------------------------------------------
// MODE 0: FP32 features; 1: bf16 hi/lo.  Feature row: [U' | V' | r' | s'] of widths Kr_pad,
// Kr_pad, Kc_pad, Kc_pad.  Frequency slot k (k >= Kc: zero padding) goes to column colmap[k] of
// the r', s' blocks: 64-wide chunks ordered so the dominant low frequencies are accumulated last
// (radius_descending_columns).
//   RINGS = false: U' = u', V' = v' per frequency (columns colmap[k]).
//   RINGS = true: v'_j(k) = sw(k) (C_j(m)^2 - mt(R)) with the ring mean mt(R) of C^2 (m = |k|^2,
//     R = k's ring; pd_finalize writes the centring sw(k) mt(R) of v and mt), so
//     sum_k u'_i v'_j = sum_R U_i(R) V_j(R) with U_i(R) = sum_{k in R} sw(k) u'_i(k) and
//     V_j(R) = C_j(m_R)^2 - mt(R): one column per ring, rings by decreasing |k|^2.  Phase 1
//     keeps sw u' of every frequency in shared memory at its position in ring order, phase 2
//     sums each ring's contiguous range.
template <int MODE, bool RINGS, int NT>
__global__ void __launch_bounds__(NT) features_kernel(
        float2* __restrict__ spec, const uint64_t* __restrict__ qfix,
        const PdDev* __restrict__ pds, const int32_t* __restrict__ img_pd,
        const int32_t* __restrict__ img_row, const FeatTables ft,
        const float* __restrict__ means,
        const uint32_t* __restrict__ scale_bits, void* __restrict__ feat_a, void* __restrict__ feat_b,
        double* __restrict__ pair_norm, float* __restrict__ ctf_out,
        float2* __restrict__ spectrum_out, int N, int Nh, int64_t Kc, int64_t Kc_pad,
        int64_t Kr, int64_t Kr_pad, int64_t mstride, CtfConst cc, int write_signed,
        int pair_loads) {
    __shared__ double red[32];
    extern __shared__ float tbuf[];          // RINGS: sw u' of every frequency (scaled)
    const int64_t img = blockIdx.x;
    const int pd = img_pd[img];
    const int64_t row = img_row[img];
    const float* mu = means + pd * mstride;
    const float sc = feature_scale_from_bits(scale_bits[pd]);
    const uint64_t qf = qfix[img];
    const float inv_nn = 1.0f / ((float)N * (float)N);
    const int64_t Kf = 2 * Kr_pad + 2 * Kc_pad;
    float2* sp = spec + img * Kc;
    KSum acc;
    auto weight = [&](int64_t k, int* m_out) {
        const int kk = (int)k;                 // < Kc_pad: 32-bit division
        const int ka = kk / Nh, kb = kk - ka * Nh;
        const int fa = min(ka, N - ka);
        *m_out = fa * fa + kb * kb;
        return (kb == 0 || ((N & 1) == 0 && kb == N / 2));     // half-plane weight 1
    };
    // features (u', v', r', s') of frequency slot k; zero for the padding k >= Kc
    auto feature = [&](int64_t k, float (&f)[4]) {
        f[0] = f[1] = f[2] = f[3] = 0.f;
        if (k >= Kc) return;
        int m;
        const bool w1 = weight(k, &m);
        const float sw = w1 ? 1.0f : 1.41421356237309505f;
        const float s2w = w1 ? 1.41421356237309505f : 2.0f;
        const float2 F = sp[k];
        if (spectrum_out) spectrum_out[img * Kc + k] = F;
        int sg;
        const float C = ctf_eval(m, qf, cc, &sg);
        const float u = sw * (F.x * F.x + F.y * F.y);
        const float v = sw * (C * C);
        const float r = s2w * C * F.x;
        const float s = s2w * C * F.y;
        const float mu_u = mu[k], mu_v = mu[Kc_pad + k];
        const float mu_r = mu[2 * Kc_pad + k], mu_s = mu[3 * Kc_pad + k];
        acc.add(mu_u * v + mu_v * u - mu_u * mu_v - mu_r * r + 0.5f * mu_r * mu_r -
                mu_s * s + 0.5f * mu_s * mu_s);
        f[0] = (u - mu_u) * sc;
        f[1] = (v - mu_v) * sc;
        f[2] = (r - mu_r) * sc;
        f[3] = (s - mu_s) * sc;
        if (RINGS) tbuf[ft.pos_of[k]] = sw * f[0];
        if (write_signed) {
            const float sgf = (float)sg * inv_nn;
            sp[k] = make_float2(sgf * F.x, sgf * F.y);
        }
    };
    // slots k, k + 1 (k even, k + 1 < Kc) with paired FP32 instructions and 16-byte spectrum /
    // 8-byte centring-vector loads (pair_loads: Kc even, so both are aligned); the same
    // operations per element as feature(), the a_i terms summed in a second compensated pair
    KSum2 acc2;
    auto feature_pair = [&](int64_t k, float (&f0)[4], float (&f1)[4]) {
        const float2 m1 = make_float2(-1.f, -1.f);
        auto sub2 = [&](float2 a, float2 b) { return __ffma2_rn(b, m1, a); };     // a - b
        int m0, mb;
        const bool w0 = weight(k, &m0), wb = weight(k + 1, &mb);
        const float2 sw = make_float2(w0 ? 1.0f : 1.41421356237309505f,
                                      wb ? 1.0f : 1.41421356237309505f);
        const float2 s2w = make_float2(w0 ? 1.41421356237309505f : 2.0f,
                                       wb ? 1.41421356237309505f : 2.0f);
        const float4 FF = *reinterpret_cast<const float4*>(sp + k);
        if (spectrum_out) *reinterpret_cast<float4*>(spectrum_out + img * Kc + k) = FF;
        int sg0, sg1;
        const float2 C = make_float2(ctf_eval(m0, qf, cc, &sg0), ctf_eval(mb, qf, cc, &sg1));
        const float2 Fx = make_float2(FF.x, FF.z), Fy = make_float2(FF.y, FF.w);
        const float2 u = __fmul2_rn(sw, __ffma2_rn(Fx, Fx, __fmul2_rn(Fy, Fy)));
        const float2 v = __fmul2_rn(sw, __fmul2_rn(C, C));
        const float2 q = __fmul2_rn(s2w, C);
        const float2 r = __fmul2_rn(q, Fx), sv = __fmul2_rn(q, Fy);
        const float2 mu_u = *reinterpret_cast<const float2*>(mu + k);
        const float2 mu_v = *reinterpret_cast<const float2*>(mu + Kc_pad + k);
        const float2 mu_r = *reinterpret_cast<const float2*>(mu + 2 * Kc_pad + k);
        const float2 mu_s = *reinterpret_cast<const float2*>(mu + 3 * Kc_pad + k);
        const float2 half = make_float2(0.5f, 0.5f);
        // mu_u (v - mu_v) + mu_v u + mu_r (mu_r / 2 - r) + mu_s (mu_s / 2 - s)
        float2 a = __fmul2_rn(mu_u, sub2(v, mu_v));
        a = __ffma2_rn(mu_v, u, a);
        a = __ffma2_rn(mu_r, sub2(__fmul2_rn(half, mu_r), r), a);
        a = __ffma2_rn(mu_s, sub2(__fmul2_rn(half, mu_s), sv), a);
        acc2.add(a);
        const float2 scv = make_float2(sc, sc);
        const float2 fu = __fmul2_rn(sub2(u, mu_u), scv), fv = __fmul2_rn(sub2(v, mu_v), scv);
        const float2 fr = __fmul2_rn(sub2(r, mu_r), scv), fs = __fmul2_rn(sub2(sv, mu_s), scv);
        f0[0] = fu.x, f0[1] = fv.x, f0[2] = fr.x, f0[3] = fs.x;
        f1[0] = fu.y, f1[1] = fv.y, f1[2] = fr.y, f1[3] = fs.y;
        if (RINGS) {
            tbuf[ft.pos_of[k]] = sw.x * fu.x;
            tbuf[ft.pos_of[k + 1]] = sw.y * fu.y;
        }
        if (write_signed) {
            const float g0 = (float)sg0 * inv_nn, g1 = (float)sg1 * inv_nn;
            *reinterpret_cast<float4*>(sp + k) =
                make_float4(g0 * FF.x, g0 * FF.y, g1 * FF.z, g1 * FF.w);
        }
    };
    auto store2 = [&](int64_t col, float a0, float a1) {     // columns col, col + 1 (col even)
        if (MODE == 1) {
            __nv_bfloat162* hi = (__nv_bfloat162*)((__nv_bfloat16*)feat_a + row * Kf);
            __nv_bfloat162* lo = (__nv_bfloat162*)((__nv_bfloat16*)feat_b + row * Kf);
            const __nv_bfloat162 h = __floats2bfloat162_rn(a0, a1);
            const float2 hf = __bfloat1622float2(h);
            hi[col >> 1] = h;
            lo[col >> 1] = __floats2bfloat162_rn(a0 - hf.x, a1 - hf.y);
        } else {
            float2* x = (float2*)((float*)feat_a + row * Kf);
            x[col >> 1] = make_float2(a0, a1);
        }
    };
    // two consecutive slots per thread: they share a 64-wide chunk, so their feature columns
    // are adjacent (col even) and each block gets one paired store
    for (int64_t k = 2 * (int64_t)threadIdx.x; k < Kc_pad; k += 2 * NT) {
        float f0[4], f1[4];
        if (pair_loads && k < Kc) {
            feature_pair(k, f0, f1);
        } else {
            feature(k, f0);
            feature(k + 1, f1);
        }
        const int64_t col = ft.colmap[k];
        if (!RINGS) {
            store2(col, f0[0], f1[0]);
            store2(Kr_pad + col, f0[1], f1[1]);
        }
        store2(2 * Kr_pad + col, f0[2], f1[2]);
        store2(2 * Kr_pad + Kc_pad + col, f0[3], f1[3]);
    }
    if (RINGS) {
        __syncthreads();
        // U(R) = sum of sw u' over the ring's members (in ring order), V(R) = C(m_R)^2 - mt(R)
        auto ring = [&](int64_t R, float* U, float* V) {
            *U = *V = 0.f;
            if (R >= Kr) return;
            const int b = ft.ring_start[R], e = ft.ring_start[R + 1];
            float su = 0.f;
            for (int i = b; i < e; ++i) su += tbuf[i];
            int sg;
            const float C = ctf_eval(ft.ring_m[R], qf, cc, &sg);
            *U = su;
            *V = (C * C - mu[4 * Kc_pad + R]) * sc;
        };
        for (int64_t R = 2 * (int64_t)threadIdx.x; R < Kr_pad; R += 2 * NT) {
            float U0, V0, U1, V1;
            ring(R, &U0, &V0);
            ring(R + 1, &U1, &V1);
            store2(R, U0, U1);
            store2(Kr_pad + R, V0, V1);
        }
    }
    const float2 a2 = acc2.value();
    const double a = block_sum_double<NT>((double)acc.value() + (double)a2.x + (double)a2.y,
                                          red);
    if (threadIdx.x == 0) pair_norm[img] = a;
    if (ctf_out) {
        float* co = ctf_out + img * (int64_t)N * N;
        for (int p = threadIdx.x; p < N * N; p += NT) {
            const int r = p / N, c = p - r * N;
            const int fa = min(r, N - r), fb = min(c, N - c);
            int sg;
            co[p] = ctf_eval(fa * fa + fb * fb, qf, cc, &sg);
        }
    }
}

// 7. averages: float C2R results -> double outputs (the reference keeps them in float64)
// with a volume mask both averages are multiplied by the PD's msk2 (reference :366-367)
__global__ void avg_store_kernel(const float* __restrict__ avg_real, double* __restrict__ img_avg,
                                 double* __restrict__ img_avg_flip, int64_t n_pd, int NN,
                                 const uint8_t* __restrict__ pd_mask) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= n_pd * NN) return;
    const int64_t pd = e / NN, p = e - pd * NN;
    const bool keep = pd_mask == nullptr || pd_mask[e] != 0;
    if (img_avg) img_avg[e] = keep ? (double)avg_real[(pd * 2) * NN + p] : 0.0;
    if (img_avg_flip) img_avg_flip[e] = keep ? (double)avg_real[(pd * 2 + 1) * NN + p] : 0.0;
}

// 8. imgAllIntensity = mean_i imgAllFlip_i^2 (reference :400)
__global__ void __launch_bounds__(256) intensity_kernel(
        const float* __restrict__ flip_imgs, const PdDev* __restrict__ pds,
        double* __restrict__ out, int NN) {
    const int p = blockIdx.y * 256 + threadIdx.x;
    const int pd = blockIdx.x;
    if (p >= NN) return;
    const PdDev d = pds[pd];
    KSum s;
    for (int i = 0; i < d.n; ++i) {
        const float v = flip_imgs[(d.img_off + i) * (int64_t)NN + p];
        s.add(v * v);
    }
    out[(int64_t)pd * NN + p] = (double)s.value() / d.n;
}


// the same for NN % 4 == 0 with four pixels per thread (16-byte loads: four times the bytes in
// flight per load; each pixel's sum in the same order)
__global__ void __launch_bounds__(256) intensity4_kernel(
        const float* __restrict__ flip_imgs, const PdDev* __restrict__ pds,
        double* __restrict__ out, int NN) {
    const int q = blockIdx.y * 256 + threadIdx.x;
    const int pd = blockIdx.x;
    if (4 * q >= NN) return;
    const PdDev d = pds[pd];
    KSum s0, s1, s2, s3;
    for (int i = 0; i < d.n; ++i) {
        const float4 v =
            reinterpret_cast<const float4*>(flip_imgs + (d.img_off + i) * (int64_t)NN)[q];
        s0.add(v.x * v.x);
        s1.add(v.y * v.y);
        s2.add(v.z * v.z);
        s3.add(v.w * v.w);
    }
    double* o = out + (int64_t)pd * NN + 4 * q;
    o[0] = (double)s0.value() / d.n;
    o[1] = (double)s1.value() / d.n;
    o[2] = (double)s2.value() / d.n;
    o[3] = (double)s3.value() / d.n;
}

}  // namespace
}  // namespace mem

// ---------------------------------------------------------------------------- launchers
namespace mem {
namespace kern {

int gather_normalize(const mem_plan& P, const mem_inputs& in, float* xbuf, uint32_t* status,
                     int64_t max_ctas, cudaStream_t s) {
    if (P.n_images == 0) return MEM_OK;
    const int64_t grid = max_ctas > 0 ? std::min<int64_t>(max_ctas, P.n_images) : P.n_images;
    if (P.N % 4 == 0)
        gather_normalize_v4_kernel<256><<<(unsigned)grid, 256, 0, s>>>(
            in.stack, in.num_stack, in.stack_index, in.flip, xbuf, P.N, status, P.n_images);
    else
        gather_normalize_kernel<256><<<(unsigned)grid, 256, 0, s>>>(
            in.stack, in.num_stack, in.stack_index, in.flip, xbuf, P.N, status, P.n_images);
    MEM_LAUNCH_CHECK();
    return MEM_OK;
}

int gather_copy(const mem_plan& P, const mem_inputs& in, float* out, uint32_t* status,
                int64_t ctas, cudaStream_t s) {
    if (P.n_images == 0) return MEM_OK;
    const int64_t grid = std::max<int64_t>(1, std::min<int64_t>(ctas, P.n_images));
    gather_copy_kernel<<<(unsigned)grid, P.host_load_threads, 0, s>>>(
            in.stack, in.num_stack, in.stack_index, P.n_images, P.N * P.N, out, status);
    MEM_LAUNCH_CHECK();
    return MEM_OK;
}

int lowpass(const mem_plan& P, float2* spec, float* gtab, cudaStream_t s) {
    const int KcN = P.N * P.Nh;
    const int64_t total = P.n_images * (int64_t)KcN;
    if (total == 0) return MEM_OK;
    const int64_t blocks = std::min<int64_t>((total + 255) / 256, (int64_t)P.num_sms * 16);
    lowpass_apply_kernel<<<(unsigned)blocks, 256, 0, s>>>(spec, gtab, total, KcN);
    MEM_LAUNCH_CHECK();
    return MEM_OK;
}

int lowpass_table(const mem_plan& P, float* gtab, cudaStream_t s) {
    const int KcN = P.N * P.Nh;
    lowpass_table_kernel<<<(KcN + 255) / 256, 256, 0, s>>>(
        gtab, P.N, P.Nh, P.params.filter_type, P.params.filter_Qc, P.params.filter_order);
    MEM_LAUNCH_CHECK();
    return MEM_OK;
}

int rot_consts(const mem_plan& P, const mem_inputs& in, const PdDev* pd_table,
               const int32_t* img_pd, void* rot_scratch, cudaStream_t s) {
    if (P.n_images == 0) return MEM_OK;
    rot_const_kernel<<<(unsigned)((P.n_images + 255) / 256), 256, 0, s>>>(
        in.psi_rad, pd_table, img_pd, static_cast<RotConst*>(rot_scratch), P.n_images, P.N);
    MEM_LAUNCH_CHECK();
    return MEM_OK;
}

int rotate(const mem_plan& P, const mem_inputs& in, float* xbuf, float* img_out,
           const PdDev* pd_table, const int32_t* img_pd, float2* spec, void* rot_scratch,
           cudaStream_t s) {
    if (P.n_images == 0) return MEM_OK;
    const int N = P.N;
    RotConst* rotc = static_cast<RotConst*>(rot_scratch);
    const int st = rot_consts(P, in, pd_table, img_pd, rot_scratch, s);
    if (st != MEM_OK) return st;
    const bool fixed_n = N == 64 || N == 128;
    if (kern::rotate_band_supported(N) &&
        ((P.rot_band >= 1 && N > kMaxSmemN) || (P.rot_band >= 2 && !fixed_n)))
        return kern::rotate_band(P, xbuf, spec, img_out, rotc, s);
    if (N > kMaxSmemN) {
        constexpr int NT = 512;
        const int nseg = std::max(1, std::min(NT / N, N / 16));
        rotate_global_kernel<NT><<<(unsigned)P.n_images, NT, 0, s>>>(
            xbuf, spec, P.Kc, img_out, rotc, N, nseg,
            (float)(1.0 / (1.0 - std::pow((double)kZ1, (double)N))));
        MEM_LAUNCH_CHECK();
        return MEM_OK;
    }
    // row strides (3-px halo): 1 and -1 mod 32, picked per rotation by its angle, where the
    // larger fits shared memory; else one odd stride for both
    int P1 = ((N + 3 + 30) / 32) * 32 + 1, Pm1 = ((N + 3 + 32) / 32) * 32 - 1;
    if ((size_t)(N + 3) * std::max(P1, Pm1) * sizeof(float) > 227 * 1024)
        P1 = Pm1 = ((N + 3) % 2 == 0) ? N + 4 : N + 3;
    const size_t smem = (size_t)(N + 3) * std::max(P1, Pm1) * sizeof(float);
    constexpr int NT = 512;
    if (N == 128 || N == 64) {
        auto kfn = N == 128 ? rotate_fixed_kernel<NT, 128> : rotate_fixed_kernel<NT, 64>;
        const size_t smem_f = (size_t)(N + 3) *
                              (N == 128 ? rot_stride<128>() : rot_stride<64>()) * sizeof(float);
        MEM_CUDA_TRY(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem_f));
        kfn<<<(unsigned)P.n_images, NT, smem_f, s>>>(xbuf, img_out, rotc);
        MEM_LAUNCH_CHECK();
        return MEM_OK;
    }
    int nseg = std::max(1, std::min(NT / N, N / 16));
    const bool exact = N < kInitTaps;
    if (exact) nseg = 1;
    const float inv1mzN = (float)(1.0 / (1.0 - std::pow((double)kZ1, (double)N)));
    const int R = NT / N;
    const int per_thread = (N + R - 1) / R;
    if (per_thread <= 32) {
        MEM_CUDA_TRY(cudaFuncSetAttribute(rotate_kernel<NT, 32>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        rotate_kernel<NT, 32><<<(unsigned)P.n_images, NT, smem, s>>>(
            xbuf, img_out, rotc, N, P1, Pm1, nseg, inv1mzN, exact ? 1 : 0);
    } else {
        MEM_CUDA_TRY(cudaFuncSetAttribute(rotate_kernel<NT, 0>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        rotate_kernel<NT, 0><<<(unsigned)P.n_images, NT, smem, s>>>(
            xbuf, img_out, rotc, N, P1, Pm1, nseg, inv1mzN, exact ? 1 : 0);
    }
    MEM_LAUNCH_CHECK();
    return MEM_OK;
}

int qfix(const mem_plan& P, const mem_inputs& in, uint64_t* qf, cudaStream_t s) {
    if (P.n_images == 0) return MEM_OK;
    qfix_kernel<<<(unsigned)((P.n_images + 255) / 256), 256, 0, s>>>(in.df, qf, P.n_images,
                                                                     P.ctf.q_scale);
    MEM_LAUNCH_CHECK();
    return MEM_OK;
}

int pd_sums(const mem_plan& P, const float2* spec, const uint64_t* qf, const SumItem* items,
            float* partial, int which, cudaStream_t s) {
    if (P.items.empty()) return MEM_OK;
    dim3 grid((unsigned)P.items.size(), (unsigned)((P.Kc + 255) / 256));
    if (which == 1)
        pd_sums_kernel<1><<<grid, 256, 0, s>>>(spec, qf, items, partial, P.N, P.Nh, P.Kc, P.ctf);
    else if (which == 2)
        pd_sums_kernel<2><<<grid, 256, 0, s>>>(spec, qf, items, partial, P.N, P.Nh, P.Kc, P.ctf);
    else
        pd_sums_kernel<3><<<grid, 256, 0, s>>>(spec, qf, items, partial, P.N, P.Nh, P.Kc, P.ctf);
    MEM_LAUNCH_CHECK();
    return MEM_OK;
}

int pd_finalize(const mem_plan& P, const float* partial, const SumItem* items,
                const int32_t* item_off, const PdDev* pds, const int32_t* ring_of, float* means,
                float2* avg_spec, uint32_t* pd_max, int mode, cudaStream_t s) {
    if (mode & 2) MEM_CUDA_TRY(cudaMemsetAsync(pd_max, 0, sizeof(uint32_t) * P.n_pd, s));
    dim3 grid((unsigned)P.n_pd, (unsigned)((P.Kc_pad + 255) / 256));
    pd_finalize_kernel<<<grid, 256, 0, s>>>(partial, items, item_off, pds,
                                            P.ring_features ? ring_of : nullptr, means, avg_spec,
                                            pd_max, P.N, P.Nh, P.Kc, P.Kc_pad,
                                            means_stride(P), mode);
    MEM_LAUNCH_CHECK();
    return MEM_OK;
}

int features(const mem_plan& P, float2* spec, const uint64_t* qf, const PdDev* pds,
             const int32_t* img_pd, const int32_t* img_row, const FeatTables& ft,
             const float* means, const uint32_t* scale_bits, void* feat_a, void* feat_b,
             double* pair_norm, float* ctf_out, float* spectrum_out, bool write_signed,
             cudaStream_t s) {
    if (P.n_images == 0) return MEM_OK;
    const size_t smem = P.ring_features ? sizeof(float) * P.Kc : 0;
    // 256 threads per image; 1024 when the ring table leaves room for fewer than three CTAs
    // per SM (large boxes: 126 KB at 250 px), so that the SM still holds 32 warps
    const bool wide = smem > 72 * 1024;
#define MEM_FEATS_NT(MODE, RINGS, NT)                                                          \
    do {                                                                                       \
        MEM_CUDA_TRY(cudaFuncSetAttribute(features_kernel<MODE, RINGS, NT>,                    \
                                          cudaFuncAttributeMaxDynamicSharedMemorySize,         \
                                          (int)smem));                                         \
        features_kernel<MODE, RINGS, NT><<<(unsigned)P.n_images, NT, smem, s>>>(               \
            spec, qf, pds, img_pd, img_row, ft, means, scale_bits, feat_a, feat_b, pair_norm,  \
            ctf_out, (float2*)spectrum_out, P.N, P.Nh, P.Kc, P.Kc_pad, P.Kr, P.Kr_pad,         \
            means_stride(P), P.ctf, write_signed ? 1 : 0, P.Kc % 2 == 0 ? 1 : 0);              \
    } while (0)
#define MEM_FEATS(MODE, RINGS)                                                                 \
    do {                                                                                       \
        if (wide) MEM_FEATS_NT(MODE, RINGS, 1024);                                             \
        else MEM_FEATS_NT(MODE, RINGS, 256);                                                   \
    } while (0)
    const bool bf16 = P.params.precision == MEM_PREC_SPLIT_BF16;
    if (P.ring_features) {
        if (bf16) MEM_FEATS(1, true);
        else MEM_FEATS(0, true);
    } else {
        if (bf16) MEM_FEATS(1, false);
        else MEM_FEATS(0, false);
    }
#undef MEM_FEATS
#undef MEM_FEATS_NT
    MEM_LAUNCH_CHECK();
    return MEM_OK;
}

int avg_store(const mem_plan& P, const float* avg_real, double* img_avg, double* img_avg_flip,
              const uint8_t* pd_mask, cudaStream_t s) {
    if (!img_avg && !img_avg_flip) return MEM_OK;
    const int NN = P.N * P.N;
    const int64_t total = (int64_t)P.n_pd * NN;
    avg_store_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(
            avg_real, img_avg, img_avg_flip, P.n_pd, NN, pd_mask);
    MEM_LAUNCH_CHECK();
    return MEM_OK;
}

int intensity(const mem_plan& P, const float* flip_imgs, const PdDev* pds, double* out,
              cudaStream_t s) {
    if (!out) return MEM_OK;
    const int NN = P.N * P.N;
    // 16-byte loads need every image to start on a 16-byte boundary
    if (NN % 4 == 0 && (reinterpret_cast<uintptr_t>(flip_imgs) & 15) == 0) {
        dim3 grid((unsigned)P.n_pd, (unsigned)((NN / 4 + 255) / 256));
        intensity4_kernel<<<grid, 256, 0, s>>>(flip_imgs, pds, out, NN);
    } else {
        dim3 grid((unsigned)P.n_pd, (unsigned)((NN + 255) / 256));
        intensity_kernel<<<grid, 256, 0, s>>>(flip_imgs, pds, out, NN);
    }
    MEM_LAUNCH_CHECK();
    return MEM_OK;
}

}  // namespace kern
}  // namespace mem
