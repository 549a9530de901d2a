// Image-side kernels of the distance stage (everything before the D contraction).
//
// Reference: modules/getDistanceCTF_local_Conj9combinedS2.py:216-400 and the helpers it calls
// (rotatefill.py, annularMask.py, ctemh_cryoFrank.py, get_wiener1 :422-430).
//
// Data layout in HBM (per call):
//   xbuf   [n_images][N][N] float   raw image (storage orientation), later scratch
//   spec   [n_images][N][N/2+1] float2   half-plane spectra (cuFFT R2C layout)
//   feats  [n_rows][4*Kc_pad]  float (FP32 form) or two bf16 matrices hi/lo (split form):
//          column blocks u' | v' | r' | s' (see features_kernel)
#include <cuda_bf16.h>
#include <algorithm>
#include <cmath>

#include "mem_internal.cuh"

namespace mem {
namespace {

constexpr float kZ1 = -0.26794919243112270f;     // sqrt(3) - 2, cubic B-spline pole
constexpr int kInitTaps = 18;                      // |z1|^18 = 5e-11

__device__ __forceinline__ float mask_ref(int r, int c, int N) {
    // annularMask.op(0, N/2, N, N) (annularMask.py:19-32): centre (N/2 - 1, N/2), radius N/2
    const float h = 0.5f * (float)N;
    const float x = (float)r - h + 1.0f, y = (float)c - h;
    return (x * x + y * y < h * h) ? 1.0f : 0.0f;
}

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
__global__ void __launch_bounds__(NT) gather_normalize_kernel(
        const float* __restrict__ stack, int64_t num_stack, const int64_t* __restrict__ sidx,
        const uint8_t* __restrict__ flip, float* __restrict__ xbuf, int N,
        uint32_t* __restrict__ status) {
    __shared__ double red[32];
    const int64_t img = blockIdx.x;
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
    const double tot = block_sum_double<NT>((double)sum.value(), red);
    const double tot2 = block_sum_double<NT>((double)sq.value(), red);
    const double mean = tot / NN;
    const double var = fmax(tot2 / NN - mean * mean, 0.0);
    const float fmean = (float)mean;
    const float inv = (float)(1.0 / sqrt(var));
    for (int p = threadIdx.x; p < NN; p += NT) {
        const int a = p / N, b = p - a * N;
        dst[p] = (src[a * N + (f ? N - 1 - b : b)] - fmean) * inv;
    }
}

// float4 variant for N % 4 == 0: one 16-byte load / store per 4 pixels of a stack row; a
// conjugate flip reverses the four lanes (the row reversal maps aligned quads to aligned quads)
template <int NT>
__global__ void __launch_bounds__(NT) gather_normalize_v4_kernel(
        const float* __restrict__ stack, int64_t num_stack, const int64_t* __restrict__ sidx,
        const uint8_t* __restrict__ flip, float* __restrict__ xbuf, int N,
        uint32_t* __restrict__ status) {
    __shared__ double red[32];
    const int64_t img = blockIdx.x;
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
    const double tot = block_sum_double<NT>((double)sum.value(), red);
    const double tot2 = block_sum_double<NT>((double)sq.value(), red);
    const double mean = tot / NN;
    const double var = fmax(tot2 / NN - mean * mean, 0.0);
    const float fmean = (float)mean;
    const float inv = (float)(1.0 / sqrt(var));
    for (int p = threadIdx.x; p < NQ; p += NT) {
        int a, b;
        const float4 v = load(p, a, b);
        dst[p] = make_float4((v.x - fmean) * inv, (v.y - fmean) * inv, (v.z - fmean) * inv,
                             (v.w - fmean) * inv);
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
// 2b. fused gather + normalisation + low-pass for power-of-two N <= 128 (one CTA per image)
//
// Same result as gather_normalize + cuFFT R2C + lowpass_apply + cuFFT C2R, with the image kept
// in shared memory: a real 2D FFT (rows: length-N/2 complex FFT of the packed pairs
// (x[2j], x[2j+1]) then the real-FFT split; columns: length-N complex FFT), the multiply by
// G/N^2, and the inverse.  Forward transforms are radix-2 decimation-in-frequency (natural in,
// bit-reversed out), inverse transforms decimation-in-time (bit-reversed in, natural out), so
// no reordering pass is needed; G is read at the bit-reversed row.  Twiddles
// exp(-2 pi i k / N), k <= N/2, come from a table computed in double on the host.
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {   // a * conj(b)
    return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}

// radix-2 DIF over `batch` signals of length 2^logL; element (b, i) at C[b*bs + i*es]
template <int NT>
__device__ void fft_dif(float2* C, int logL, int batch, int bs, int es, const float2* tw, int logN,
                        bool lanes_on_batch) {
    const int L = 1 << logL, half = L >> 1;
    for (int lh = logL - 1; lh >= 0; --lh) {
        const int h = 1 << lh;
        const int tstride = logN - lh - 1;            // twiddle index step N / (2h)
        for (int t = threadIdx.x; t < batch * half; t += NT) {
            int b, q;
            if (lanes_on_batch) { b = t % batch; q = t / batch; }
            else { b = t >> (logL - 1); q = t & (half - 1); }
            const int j = q & (h - 1);
            const int i0 = ((q >> lh) << (lh + 1)) + j;
            float2* p0 = C + b * bs + i0 * es;
            float2* p1 = p0 + h * es;
            const float2 u = *p0, v = *p1;
            *p0 = make_float2(u.x + v.x, u.y + v.y);
            *p1 = cmul(make_float2(u.x - v.x, u.y - v.y), tw[j << tstride]);
        }
        __syncthreads();
    }
}

// radix-2 DIT inverse (conjugate twiddles, unnormalised), bit-reversed in, natural out
template <int NT>
__device__ void fft_dit_inv(float2* C, int logL, int batch, int bs, int es, const float2* tw,
                            int logN, bool lanes_on_batch) {
    const int L = 1 << logL, half = L >> 1;
    for (int lh = 0; lh < logL; ++lh) {
        const int h = 1 << lh;
        const int tstride = logN - lh - 1;
        for (int t = threadIdx.x; t < batch * half; t += NT) {
            int b, q;
            if (lanes_on_batch) { b = t % batch; q = t / batch; }
            else { b = t >> (logL - 1); q = t & (half - 1); }
            const int j = q & (h - 1);
            const int i0 = ((q >> lh) << (lh + 1)) + j;
            float2* p0 = C + b * bs + i0 * es;
            float2* p1 = p0 + h * es;
            const float2 u = *p0;
            const float2 v = cmulc(*p1, tw[j << tstride]);
            *p0 = make_float2(u.x + v.x, u.y + v.y);
            *p1 = make_float2(u.x - v.x, u.y - v.y);
        }
        __syncthreads();
    }
}

__device__ __forceinline__ int bitrev(int k, int bits) { return (int)(__brev((unsigned)k) >> (32 - bits)); }

template <int NT, int LOGN>
__global__ void __launch_bounds__(NT) lowpass_fused_kernel(
        const float* __restrict__ stack, int64_t num_stack, const int64_t* __restrict__ sidx,
        const uint8_t* __restrict__ flip, const float* __restrict__ gtab,
        const float2* __restrict__ twid, float* __restrict__ xbuf, uint32_t* __restrict__ status) {
    constexpr int N = 1 << LOGN, H = N / 2, LOGH = LOGN - 1, RS = H + 1;   // row stride (float2)
    constexpr int NN = N * N, NQ = NN / 4;
    constexpr int PAIRS = N * (H / 2 + 1);                   // (row, k) pairs of the real split
    constexpr int PER = (PAIRS + NT - 1) / NT;
    extern __shared__ float2 C[];                            // [N][H+1]
    __shared__ float2 tw[H + 1];
    __shared__ double red[32];
    const int64_t img = blockIdx.x;
    const int64_t s = sidx[img];
    float* dst = xbuf + img * (int64_t)NN;
    if (s < 0 || s >= num_stack) {
        if (threadIdx.x == 0) atomicOr(status, 2u);
        for (int p = threadIdx.x; p < NN; p += NT) dst[p] = __int_as_float(0x7fc00000);
        return;
    }
    for (int k = threadIdx.x; k <= H; k += NT) tw[k] = twid[k];
    const bool f = flip[img] != 0;
    const float4* src = reinterpret_cast<const float4*>(stack + s * (int64_t)NN);
    auto load = [&](int p, int& a, int& b) -> float4 {
        const int e = 4 * p;
        a = e >> LOGN;
        b = e & (N - 1);
        float4 v = src[(a * N + (f ? N - 4 - b : b)) >> 2];
        if (f) v = make_float4(v.w, v.z, v.y, v.x);
        return v;
    };
    // background statistics (reference :277-281)
    KSum sum, sq;
    for (int p = threadIdx.x; p < NQ; p += NT) {
        int a, b;
        const float4 v = load(p, a, b);
        const float vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float bg = vv[j] * (1.0f - mask_ref(b + j, a, N));
            sum.add(bg);
            sq.add(bg * bg);
        }
    }
    const double tot = block_sum_double<NT>((double)sum.value(), red);
    const double tot2 = block_sum_double<NT>((double)sq.value(), red);
    const double mean = tot / NN;
    const float fmean = (float)mean;
    const float inv = (float)(1.0 / sqrt(fmax(tot2 / NN - mean * mean, 0.0)));
    // normalised storage-orientation rows as packed complex pairs
    for (int p = threadIdx.x; p < NQ; p += NT) {
        int a, b;
        const float4 v = load(p, a, b);
        float2* row = C + a * RS + (b >> 1);
        row[0] = make_float2((v.x - fmean) * inv, (v.y - fmean) * inv);
        row[1] = make_float2((v.z - fmean) * inv, (v.w - fmean) * inv);
    }
    __syncthreads();
    // rows: length-H complex FFT, then the real split X[k], k = 0..H
    fft_dif<NT>(C, LOGH, N, RS, 1, tw, LOGN, false);
    {
        float2 o0[PER], o1[PER];
#pragma unroll
        for (int u = 0; u < PER; ++u) {
            const int t = threadIdx.x + u * NT;
            if (t >= PAIRS) break;
            const int r = t / (H / 2 + 1), k = t - r * (H / 2 + 1);
            const float2* row = C + r * RS;
            const float2 zk = row[bitrev(k & (H - 1), LOGH)];
            const float2 zm = row[bitrev((H - k) & (H - 1), LOGH)];
            // X[k] = (zk + conj zm)/2 - i w_k (zk - conj zm)/2,  w_k = exp(-2 pi i k / N)
            const float2 e = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y - zm.y));
            const float2 d = make_float2(0.5f * (zk.x - zm.x), 0.5f * (zk.y + zm.y));
            const float2 wd = cmul(tw[k], d);
            o0[u] = make_float2(e.x + wd.y, e.y - wd.x);
            // X[H-k] from the same pair: (zm + conj zk)/2 - i w_{H-k} (zm - conj zk)/2
            const float2 e2 = make_float2(0.5f * (zm.x + zk.x), 0.5f * (zm.y - zk.y));
            const float2 d2 = make_float2(0.5f * (zm.x - zk.x), 0.5f * (zm.y + zk.y));
            const float2 wd2 = cmul(tw[H - k], d2);
            o1[u] = make_float2(e2.x + wd2.y, e2.y - wd2.x);
        }
        __syncthreads();
#pragma unroll
        for (int u = 0; u < PER; ++u) {
            const int t = threadIdx.x + u * NT;
            if (t >= PAIRS) break;
            const int r = t / (H / 2 + 1), k = t - r * (H / 2 + 1);
            float2* row = C + r * RS;
            row[k] = o0[u];
            row[H - k] = o1[u];
        }
        __syncthreads();
    }
    // columns: length-N complex FFT (rows come out bit-reversed), multiply by G/N^2, inverse
    fft_dif<NT>(C, LOGN, RS, 1, RS, tw, LOGN, true);
    for (int e = threadIdx.x; e < N * RS; e += NT) {
        const int i = e / RS, kc = e - i * RS;
        const float g = gtab[bitrev(i, LOGN) * RS + kc];
        C[e] = make_float2(C[e].x * g, C[e].y * g);
    }
    __syncthreads();
    fft_dit_inv<NT>(C, LOGN, RS, 1, RS, tw, LOGN, true);
    // rows: inverse real split Z[k] = (X[k] + conj X[H-k]) + i conj(w_k)(X[k] - conj X[H-k]),
    // stored bit-reversed for the inverse DIT, then the length-H inverse FFT
    {
        float2 o0[PER], o1[PER];
#pragma unroll
        for (int u = 0; u < PER; ++u) {
            const int t = threadIdx.x + u * NT;
            if (t >= PAIRS) break;
            const int r = t / (H / 2 + 1), k = t - r * (H / 2 + 1);
            const float2* row = C + r * RS;
            const float2 xk = row[k], xm = row[H - k];
            const float2 e = make_float2(xk.x + xm.x, xk.y - xm.y);
            const float2 d = make_float2(xk.x - xm.x, xk.y + xm.y);
            const float2 wd = cmulc(d, tw[k]);
            o0[u] = make_float2(e.x - wd.y, e.y + wd.x);
            const float2 e2 = make_float2(xm.x + xk.x, xm.y - xk.y);
            const float2 d2 = make_float2(xm.x - xk.x, xm.y + xk.y);
            const float2 wd2 = cmulc(d2, tw[H - k]);
            o1[u] = make_float2(e2.x - wd2.y, e2.y + wd2.x);
        }
        __syncthreads();
#pragma unroll
        for (int u = 0; u < PER; ++u) {
            const int t = threadIdx.x + u * NT;
            if (t >= PAIRS) break;
            const int r = t / (H / 2 + 1), k = t - r * (H / 2 + 1);
            float2* row = C + r * RS;
            if (k < H) row[bitrev(k, LOGH)] = o0[u];
            if (k > 0 && k < H) row[bitrev(H - k, LOGH)] = o1[u];
        }
        __syncthreads();
    }
    fft_dit_inv<NT>(C, LOGH, N, RS, 1, tw, LOGN, false);
    for (int p = threadIdx.x; p < N * H; p += NT) {
        const int a = p >> LOGH, j = p & (H - 1);
        reinterpret_cast<float2*>(dst)[p] = C[a * RS + j];
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
// z1 = sqrt(3) - 2, each row (then column) split into segments whose start values are the
// truncated geometric sums over the previous kInitTaps samples (exact to |z1|^24).
// Sample coordinates are computed in 64-bit fixed point (32 fractional bits).
// ------------------------------------------------------------------------------------------
struct RotConst {
    int64_t bx, by, rc, rs;   // fixed-point x = bx + r rc + c rs, y = by - r rs + c rc
};

__device__ __forceinline__ RotConst make_rot(double cs, double sn, int N) {
    const double c0 = 0.5 * (N - 1);
    const double two32 = 4294967296.0;
    RotConst R;
    R.bx = __double2ll_rn(c0 * (1.0 - cs - sn) * two32);
    R.by = __double2ll_rn(c0 * (1.0 + sn - cs) * two32);
    R.rc = __double2ll_rn(cs * two32);
    R.rs = __double2ll_rn(sn * two32);
    return R;
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

__device__ __forceinline__ void bspline_w(float t, float w[4]) {
    const float u = 1.0f - t;
    const float t2 = t * t, u2 = u * u;
    w[0] = (1.0f / 6.0f) * u2 * u;
    w[3] = (1.0f / 6.0f) * t2 * t;
    w[1] = (2.0f / 3.0f) - t2 * (1.0f - 0.5f * t);
    w[2] = (2.0f / 3.0f) - u2 * (1.0f - 0.5f * u);
}

// wrapped index of i in [-N, 2N)
__device__ __forceinline__ int wrapN(int i, int N) {
    i += (i < 0) ? N : 0;
    return i - ((i >= N) ? N : 0);
}

// The coefficient image sits in smem with a 3-pixel periodic halo: rows/columns N..N+2 repeat
// 0..2, so the 4x4 taps at (r0..r0+3, c0..c0+3), r0, c0 in [0, N), need no further wrapping.
template <int NT>
__device__ __forceinline__ void fill_halo(float* s, int N, int P) {
    __syncthreads();
    for (int p = threadIdx.x; p < 3 * N; p += NT) {
        const int r = p / N, c = p - r * N;
        s[(N + r) * P + c] = s[r * P + c];
    }
    __syncthreads();
    for (int p = threadIdx.x; p < 3 * (N + 3); p += NT) {
        const int r = p / 3, c = p - r * 3;
        s[r * P + N + c] = s[r * P + c];
    }
    __syncthreads();
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
// sample coordinates advance by a constant fixed-point step.
template <int NT, int MAXV>
__global__ void __launch_bounds__(NT) rotate_kernel(
        float* __restrict__ xbuf, float* __restrict__ img_out, const double* __restrict__ psi_rad,
        const PdDev* __restrict__ pds, const int32_t* __restrict__ img_pd, int N, int P,
        int nseg, float inv1mzN, int exact_init) {
    extern __shared__ float s[];
    __shared__ RotConst rot[2];
    const int64_t img = blockIdx.x;
    const int NN = N * N;
    float* xi = xbuf + img * (int64_t)NN;
    const int R = NT / N;                       // rows per pass
    const int c = threadIdx.x % N;
    const int r0 = threadIdx.x / N;
    const bool active = r0 < R;
    if (threadIdx.x == 0) {
        // first rotation: rotatefill(img, -(180/pi) Psi) -> t = deg2rad(that)
        const double ang = -(180.0 / 3.141592653589793) * psi_rad[img];
        const double t = ang * (3.141592653589793 / 180.0);
        rot[0] = make_rot(cos(t), sin(t), N);
        const PdDev& pd = pds[img_pd[img]];
        rot[1] = make_rot(pd.rot2_cos, pd.rot2_sin, N);
    }
    // load (storage orientation) into smem in reference orientation, times the mask
    for (int p = threadIdx.x; p < NN; p += NT) {
        const int a = p / N, b = p - a * N;
        s[b * P + a] = xi[p] * mask_ref(b, a, N);
    }
    __syncthreads();
    prefilter_axis<NT>(s, N, P, 0, nseg, inv1mzN, exact_init != 0);
    prefilter_axis<NT>(s, N, P, 1, nseg, inv1mzN, exact_init != 0);
    fill_halo<NT>(s, N, P);
    float keep[MAXV > 0 ? MAXV : 1];
    {
        const RotConst Q = rot[0];
        int64_t X = Q.bx + (int64_t)r0 * Q.rc + (int64_t)c * Q.rs;
        int64_t Y = Q.by - (int64_t)r0 * Q.rs + (int64_t)c * Q.rc;
        const int64_t dX = (int64_t)R * Q.rc, dY = -(int64_t)R * Q.rs;
        if (MAXV > 0) {
#pragma unroll
            for (int k = 0; k < MAXV; ++k) {
                const int r = r0 + k * R;
                if (active && r < N) keep[k] = sample_at(s, N, P, X, Y);
                X += dX;
                Y += dY;
            }
        } else if (active) {
            for (int r = r0; r < N; r += R, X += dX, Y += dY) xi[r * N + c] = sample_at(s, N, P, X, Y);
        }
    }
    __syncthreads();
    if (MAXV > 0) {
#pragma unroll
        for (int k = 0; k < MAXV; ++k) {
            const int r = r0 + k * R;
            if (active && r < N) s[r * P + c] = keep[k];
        }
    } else {
        for (int p = threadIdx.x; p < NN; p += NT) {
            const int r = p / N, cc = p - r * N;
            s[r * P + cc] = xi[p];
        }
    }
    __syncthreads();
    prefilter_axis<NT>(s, N, P, 0, nseg, inv1mzN, exact_init != 0);
    prefilter_axis<NT>(s, N, P, 1, nseg, inv1mzN, exact_init != 0);
    fill_halo<NT>(s, N, P);
    if (!active) return;
    const RotConst Q = rot[1];
    int64_t X = Q.bx + (int64_t)r0 * Q.rc + (int64_t)c * Q.rs;
    int64_t Y = Q.by - (int64_t)r0 * Q.rs + (int64_t)c * Q.rc;
    const int64_t dX = (int64_t)R * Q.rc, dY = -(int64_t)R * Q.rs;
    float* out = img_out + img * (int64_t)NN;
    for (int r = r0; r < N; r += R, X += dX, Y += dY) out[r * N + c] = sample_at(s, N, P, X, Y);
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
        const double* __restrict__ psi_rad, const PdDev* __restrict__ pds,
        const int32_t* __restrict__ img_pd, int N, int nseg, float inv1mzN) {
    __shared__ RotConst rot[2];
    const int64_t img = blockIdx.x;
    const int NN = N * N;
    float* B = xbuf + img * (int64_t)NN;
    float* A = reinterpret_cast<float*>(spec + img * Kc);
    if (threadIdx.x == 0) {
        const double ang = -(180.0 / 3.141592653589793) * psi_rad[img];
        const double t = ang * (3.141592653589793 / 180.0);
        rot[0] = make_rot(cos(t), sin(t), N);
        const PdDev& pd = pds[img_pd[img]];
        rot[1] = make_rot(pd.rot2_cos, pd.rot2_sin, N);
    }
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

__device__ __forceinline__ float ctf_eval(int m, uint64_t qf, const CtfConst& cc, int* sgn) {
    const uint64_t mm = (uint64_t)m;
    const uint64_t ph = cc.p_fix * (mm * mm) - qf * mm - cc.d_fix;
    const int64_t sph = (int64_t)ph;
    *sgn = (sph > 0) - (sph < 0);
    const float cyc = (float)sph * 5.421010862427522e-20f;   // 2^-64
    float v = cc.amp * sinpif(2.0f * cyc);
    if (cc.env_c != 0.0f) v *= expf(-cc.env_c * (float)m);
    return v;
}

// ------------------------------------------------------------------------------------------
// 4. per-PD sums over images (partial, one item = up to kSumChunk images of one PD)
//    S0 = sum C^2, S1/S2 = sum C F, S3/S4 = sum sign(C) F, S5 = sum |F|^2
// ------------------------------------------------------------------------------------------
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
        KSum s0, s1, s2, s3, s4, s5;
        for (int64_t i = it.img_begin; i < it.img_end; ++i) {
            const float2 F = spec[i * Kc + k];
            int sg;
            const float C = ctf_eval(m, qfix[i], cc, &sg);
            s0.add(C * C);
            s1.add(C * F.x);
            s2.add(C * F.y);
            s3.add(sg > 0 ? F.x : (sg < 0 ? -F.x : 0.f));
            s4.add(sg > 0 ? F.y : (sg < 0 ? -F.y : 0.f));
            s5.add(F.x * F.x + F.y * F.y);
        }
        float* out = partial + (int64_t)blockIdx.x * 6 * Kc + k;
        out[0 * Kc] = s0.value();
        out[1 * Kc] = s1.value();
        out[2 * Kc] = s2.value();
        out[3 * Kc] = s3.value();
        out[4 * Kc] = s4.value();
        out[5 * Kc] = s5.value();
    }
}

// 5. finalize: FP64 sum over the PD's items; centring vectors, average spectra, scale
__global__ void __launch_bounds__(256) pd_finalize_kernel(
        const float* __restrict__ partial, const SumItem* __restrict__ items,
        const int32_t* __restrict__ item_off, const PdDev* __restrict__ pds,
        float* __restrict__ means, float2* __restrict__ avg_spec, uint32_t* __restrict__ pd_max,
        int N, int Nh, int64_t Kc, int64_t Kc_pad, int64_t mstride) {
    const int64_t k = blockIdx.y * 256ll + threadIdx.x;
    const int pd = blockIdx.x;
    if (k >= Kc_pad) return;
    float* mu = means + pd * mstride;
    if (k >= Kc) {
        mu[k] = mu[Kc_pad + k] = mu[2 * Kc_pad + k] = mu[3 * Kc_pad + k] = 0.f;
        return;
    }
    double S[6] = {0, 0, 0, 0, 0, 0};
    for (int it = item_off[pd]; it < item_off[pd + 1]; ++it) {
        const float* p = partial + (int64_t)it * 6 * Kc + k;
#pragma unroll
        for (int j = 0; j < 6; ++j) S[j] += (double)p[j * Kc];
    }
    const int n = pds[pd].n;
    const int kb = (int)(k % Nh);
    const double w = (kb == 0 || (N % 2 == 0 && kb == N / 2)) ? 1.0 : 2.0;
    const double sw = sqrt(w), s2w = sqrt(2.0 * w);
    const float mu_u = (float)(sw * S[5] / n), mu_v = (float)(sw * S[0] / n);
    const float mu_r = (float)(s2w * S[1] / n), mu_s = (float)(s2w * S[2] / n);
    mu[k] = mu_u;
    mu[Kc_pad + k] = mu_v;
    mu[2 * Kc_pad + k] = mu_r;
    mu[3 * Kc_pad + k] = mu_s;
    const float mx = fmaxf(fmaxf(fabsf(mu_u), fabsf(mu_v)), fmaxf(fabsf(mu_r), fabsf(mu_s)));
    atomicMax(pd_max + pd, __float_as_uint(mx));
    // Wiener average (reference :353-366): sum_i F_i C_i / -(sum C^2 + 1/5), / N^2 (ifft2), / n
    const double NN = (double)N * N;
    const double wd = -(S[0] + 0.2);
    float2* av = avg_spec + (int64_t)pd * 2 * Kc;
    av[k] = make_float2((float)(S[1] / wd / NN / n), (float)(S[2] / wd / NN / n));
    // phase-flipped average (:346-348, :367): sum_i sign(C_i) F_i / N^2 / n
    av[Kc + k] = make_float2((float)(S[3] / NN / n), (float)(S[4] / NN / n));
}

// ------------------------------------------------------------------------------------------
// 6. features of one image (one CTA per image)
//   u = sqrt(w)|F|^2, v = sqrt(w) C^2, r = sqrt(2w) C Re F, s = sqrt(2w) C Im F, w the
//   half-plane weight; with x' = x - mean_PD(x):
//     D_ij = a_i + a_j + [u'_i.v'_j + v'_i.u'_j - r'_i.r'_j - s'_i.s'_j]
//     a_i  = sum_k (mu_u v_ik + mu_v u_ik - mu_u mu_v - mu_r r_ik + mu_r^2/2 - mu_s s_ik + mu_s^2/2)
//   (an exact rewrite of D_ij = sum_k |C_j F_i - C_i F_j|^2 for any centring vector mu).
//   Features are written scaled by the PD's power of two; a_i in FP64 unscaled.
//   The spectrum is overwritten with sign(C) F / N^2 (input of the phase-flip inverse FFT).
// ------------------------------------------------------------------------------------------
// MODE 0: FP32 features; 1: bf16 hi/lo.  Frequency slot k (k >= Kc: zero padding) goes to
// feature column colmap[k]: 64-wide chunks ordered so the dominant low frequencies are
// accumulated last (radius_descending_columns).
template <int MODE>
__global__ void __launch_bounds__(256) features_kernel(
        float2* __restrict__ spec, const uint64_t* __restrict__ qfix,
        const PdDev* __restrict__ pds, const int32_t* __restrict__ img_pd,
        const int32_t* __restrict__ img_row, const int32_t* __restrict__ colmap,
        const float* __restrict__ means,
        const uint32_t* __restrict__ scale_bits, void* __restrict__ feat_a, void* __restrict__ feat_b,
        double* __restrict__ pair_norm, float* __restrict__ ctf_out,
        float2* __restrict__ spectrum_out, int N, int Nh, int64_t Kc, int64_t Kc_pad,
        int64_t mstride, CtfConst cc) {
    __shared__ double red[32];
    const int64_t img = blockIdx.x;
    const int pd = img_pd[img];
    const int64_t row = img_row[img];
    const float* mu = means + pd * mstride;
    const float sc = feature_scale_from_bits(scale_bits[pd]);
    const uint64_t qf = qfix[img];
    const float inv_nn = 1.0f / ((float)N * (float)N);
    const int64_t K4 = 4 * Kc_pad;
    float2* sp = spec + img * Kc;
    KSum acc;
    for (int64_t k = threadIdx.x; k < Kc_pad; k += 256) {
        float fu = 0.f, fv = 0.f, fr = 0.f, fs = 0.f;
        const int64_t col = colmap[k];
        if (k < Kc) {
            const int ka = (int)(k / Nh), kb = (int)(k - (int64_t)ka * Nh);
            const int fa = min(ka, N - ka);
            const int m = fa * fa + kb * kb;
            const bool w1 = (kb == 0 || ((N & 1) == 0 && kb == N / 2));
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
            fu = (u - mu_u) * sc;
            fv = (v - mu_v) * sc;
            fr = (r - mu_r) * sc;
            fs = (s - mu_s) * sc;
            const float sgf = (float)sg * inv_nn;
            sp[k] = make_float2(sgf * F.x, sgf * F.y);
        }
        const float vals[4] = {fu, fv, fr, fs};
        if (MODE == 1) {
            __nv_bfloat16* hi = (__nv_bfloat16*)feat_a + row * K4;
            __nv_bfloat16* lo = (__nv_bfloat16*)feat_b + row * K4;
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const __nv_bfloat16 h = __float2bfloat16_rn(vals[b]);
                hi[b * Kc_pad + col] = h;
                lo[b * Kc_pad + col] = __float2bfloat16_rn(vals[b] - __bfloat162float(h));
            }
        } else {
            float* x = (float*)feat_a + row * K4;
#pragma unroll
            for (int b = 0; b < 4; ++b) x[b * Kc_pad + col] = vals[b];
        }
    }
    const double a = block_sum_double<256>((double)acc.value(), red);
    if (threadIdx.x == 0) pair_norm[img] = a;
    if (ctf_out) {
        float* co = ctf_out + img * (int64_t)N * N;
        for (int p = threadIdx.x; p < N * N; p += 256) {
            const int r = p / N, c = p - r * N;
            const int fa = min(r, N - r), fb = min(c, N - c);
            int sg;
            co[p] = ctf_eval(fa * fa + fb * fb, qf, cc, &sg);
        }
    }
}

// 7. averages: float C2R results -> double outputs (the reference keeps them in float64)
__global__ void avg_store_kernel(const float* __restrict__ avg_real, double* __restrict__ img_avg,
                                 double* __restrict__ img_avg_flip, int64_t n_pd, int NN) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= n_pd * NN) return;
    const int64_t pd = e / NN, p = e - pd * NN;
    if (img_avg) img_avg[e] = (double)avg_real[(pd * 2) * NN + p];
    if (img_avg_flip) img_avg_flip[e] = (double)avg_real[(pd * 2 + 1) * NN + p];
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

}  // namespace
}  // namespace mem

// ---------------------------------------------------------------------------- launchers
namespace mem {
namespace kern {

int gather_normalize(const mem_plan& P, const mem_inputs& in, float* xbuf, uint32_t* status,
                     cudaStream_t s) {
    if (P.n_images == 0) return MEM_OK;
    if (P.N % 4 == 0)
        gather_normalize_v4_kernel<256><<<(unsigned)P.n_images, 256, 0, s>>>(
            in.stack, in.num_stack, in.stack_index, in.flip, xbuf, P.N, status);
    else
        gather_normalize_kernel<256><<<(unsigned)P.n_images, 256, 0, s>>>(
            in.stack, in.num_stack, in.stack_index, in.flip, xbuf, P.N, status);
    MEM_LAUNCH_CHECK();
    return MEM_OK;
}

int lowpass(const mem_plan& P, float2* spec, float* gtab, cudaStream_t s) {
    const int KcN = P.N * P.Nh;
    lowpass_table_kernel<<<(KcN + 255) / 256, 256, 0, s>>>(
        gtab, P.N, P.Nh, P.params.filter_type, P.params.filter_Qc, P.params.filter_order);
    MEM_LAUNCH_CHECK();
    const int64_t total = P.n_images * (int64_t)KcN;
    if (total == 0) return MEM_OK;
    const int64_t blocks = std::min<int64_t>((total + 255) / 256, (int64_t)P.num_sms * 16);
    lowpass_apply_kernel<<<(unsigned)blocks, 256, 0, s>>>(spec, gtab, total, KcN);
    MEM_LAUNCH_CHECK();
    return MEM_OK;
}

bool lowpass_fused_supported(const mem_plan& P) {
    const int N = P.N;
    return N >= 16 && N <= 128 && (N & (N - 1)) == 0;
}

int lowpass_fused(const mem_plan& P, const mem_inputs& in, const float* gtab,
                  const float2* twid, float* xbuf, uint32_t* status, cudaStream_t s) {
    if (P.n_images == 0) return MEM_OK;
    constexpr int NT = 512;
    const size_t smem = (size_t)P.N * (P.N / 2 + 1) * sizeof(float2);
#define MEM_LPF(LOGN)                                                                              do {                                                                                               MEM_CUDA_TRY(cudaFuncSetAttribute(lowpass_fused_kernel<NT, LOGN>,                                                                cudaFuncAttributeMaxDynamicSharedMemorySize,                                                   (int)smem));                                                 lowpass_fused_kernel<NT, LOGN><<<(unsigned)P.n_images, NT, smem, s>>>(                             in.stack, in.num_stack, in.stack_index, in.flip, gtab, twid, xbuf, status);            } while (0)
    switch (P.N) {
        case 16: MEM_LPF(4); break;
        case 32: MEM_LPF(5); break;
        case 64: MEM_LPF(6); break;
        case 128: MEM_LPF(7); break;
        default: return MEM_ERR_UNSUPPORTED;
    }
#undef MEM_LPF
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

int rotate(const mem_plan& P, const mem_inputs& in, float* xbuf, float* img_out,
           const PdDev* pd_table, const int32_t* img_pd, float2* spec, cudaStream_t s) {
    if (P.n_images == 0) return MEM_OK;
    const int N = P.N;
    if (N > kMaxSmemN) {
        constexpr int NT = 512;
        const int nseg = std::max(1, std::min(NT / N, N / 16));
        rotate_global_kernel<NT><<<(unsigned)P.n_images, NT, 0, s>>>(
            xbuf, spec, P.Kc, img_out, in.psi_rad, pd_table, img_pd, N, nseg,
            (float)(1.0 / (1.0 - std::pow((double)kZ1, (double)N))));
        MEM_LAUNCH_CHECK();
        return MEM_OK;
    }
    const int Pst = ((N + 3) % 2 == 0) ? N + 4 : N + 3;     // odd row stride, 3-px halo
    const size_t smem = (size_t)(N + 3) * Pst * sizeof(float);
    constexpr int NT = 512;
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
            xbuf, img_out, in.psi_rad, pd_table, img_pd, N, Pst, nseg, inv1mzN, exact ? 1 : 0);
    } else {
        MEM_CUDA_TRY(cudaFuncSetAttribute(rotate_kernel<NT, 0>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        rotate_kernel<NT, 0><<<(unsigned)P.n_images, NT, smem, s>>>(
            xbuf, img_out, in.psi_rad, pd_table, img_pd, N, Pst, nseg, inv1mzN, exact ? 1 : 0);
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
            float* partial, cudaStream_t s) {
    if (P.items.empty()) return MEM_OK;
    dim3 grid((unsigned)P.items.size(), (unsigned)((P.Kc + 255) / 256));
    pd_sums_kernel<<<grid, 256, 0, s>>>(spec, qf, items, partial, P.N, P.Nh, P.Kc, P.ctf);
    MEM_LAUNCH_CHECK();
    return MEM_OK;
}

int pd_finalize(const mem_plan& P, const float* partial, const SumItem* items,
                const int32_t* item_off, const PdDev* pds, float* means, float2* avg_spec,
                uint32_t* pd_max, cudaStream_t s) {
    MEM_CUDA_TRY(cudaMemsetAsync(pd_max, 0, sizeof(uint32_t) * P.n_pd, s));
    dim3 grid((unsigned)P.n_pd, (unsigned)((P.Kc_pad + 255) / 256));
    pd_finalize_kernel<<<grid, 256, 0, s>>>(partial, items, item_off, pds, means, avg_spec,
                                            pd_max, P.N, P.Nh, P.Kc, P.Kc_pad,
                                            means_stride(P));
    MEM_LAUNCH_CHECK();
    return MEM_OK;
}

int features(const mem_plan& P, float2* spec, const uint64_t* qf, const PdDev* pds,
             const int32_t* img_pd, const int32_t* img_row, const int32_t* colmap,
             const float* means, const uint32_t* scale_bits, void* feat_a, void* feat_b,
             double* pair_norm, float* ctf_out, float* spectrum_out, cudaStream_t s) {
    if (P.n_images == 0) return MEM_OK;
#define MEM_FEATS(MODE)                                                                        \
    features_kernel<MODE><<<(unsigned)P.n_images, 256, 0, s>>>(                                \
        spec, qf, pds, img_pd, img_row, colmap, means, scale_bits, feat_a, feat_b, pair_norm,  \
        ctf_out, (float2*)spectrum_out, P.N, P.Nh, P.Kc, P.Kc_pad, means_stride(P), P.ctf)
    if (P.params.precision == MEM_PREC_SPLIT_BF16)
        MEM_FEATS(1);
    else
        MEM_FEATS(0);
#undef MEM_FEATS
    MEM_LAUNCH_CHECK();
    return MEM_OK;
}

int avg_store(const mem_plan& P, const float* avg_real, double* img_avg, double* img_avg_flip,
              cudaStream_t s) {
    if (!img_avg && !img_avg_flip) return MEM_OK;
    const int NN = P.N * P.N;
    const int64_t total = (int64_t)P.n_pd * NN;
    avg_store_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(avg_real, img_avg,
                                                                    img_avg_flip, P.n_pd, NN);
    MEM_LAUNCH_CHECK();
    return MEM_OK;
}

int intensity(const mem_plan& P, const float* flip_imgs, const PdDev* pds, double* out,
              cudaStream_t s) {
    if (!out) return MEM_OK;
    const int NN = P.N * P.N;
    dim3 grid((unsigned)P.n_pd, (unsigned)((NN + 255) / 256));
    intensity_kernel<<<grid, 256, 0, s>>>(flip_imgs, pds, out, NN);
    MEM_LAUNCH_CHECK();
    return MEM_OK;
}

}  // namespace kern
}  // namespace mem
