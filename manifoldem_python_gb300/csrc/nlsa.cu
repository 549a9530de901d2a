// NLSA snapshot stage of one PD (reference modules/NLSA.py:23-158, get_wiener.py:9-21): the
// concatenated-distance matrix ConD and the snapshot matrix A that NLSA.op builds from the PD's
// images before its small SVD.
//
// ConD = sum_{i < c} DD[i:i+m, i:i+m] (NLSA.py:31-34) is a band sum along the diagonals, one
// thread per element, added in the reference's order (bit-identical).
//
// A (NLSA.py:63-86): block ii of A is tmp_ii mu_psi, where column i of tmp_ii is the masked,
// Wiener-filtered image j = c - ii + i - 1,
//     msk2 * Re ifft2(F_j C_j / wd_i),   wd_i = sum_{t=i+1}^{i+c} C_t^2 + 1/5.
// The reference runs c (num - c) forward/inverse transform pairs.  Both the inverse transform and
// the product with mu_psi are linear, and mu_psi is real, so
//     A_ii[:, l] = msk2 * Re ifft2( sum_i F_j C_j / wd_i mu_psi[i, l] ),
// which needs num forward transforms, one banded correlation in the frequency domain and
// c * n_modes inverse transforms.  C_j and wd_i are even in frequency, so F_j C_j / wd_i is
// Hermitian and the sum runs over the half-plane spectra [N][N/2+1] of an R2C transform.
//
// The correlation G[ii][l](k) = sum_i h_{i+c-1-ii}(k) g_{i,l}(k), h_j = F_j C_j,
// g_{i,l} = mu_psi[i,l] / wd_i(k), is done per frequency: a thread owns one k, kLags consecutive
// lags ii and kModes modes, keeps the window h_{i+c-1-ii0} .. h_{i+c-1-ii0-kLags+1} in registers
// (one new spectrum element per step i) and accumulates kLags x kModes complex sums with paired
// FP32 FMAs.  The i range is split into S chunks (grid z) whose partial sums are added in a fixed
// order afterwards.  The unfiltered 'cuti' branch (NLSA.py:54-55) is the same correlation of the
// raw pixels with weight 1.
#include <algorithm>
#include <cmath>

#include "mem_internal.cuh"

namespace mem {
namespace {

constexpr int kModes = 8;          // modes per correlation pass
constexpr int kLags = 4;           // lags ii per thread
constexpr int kCorrThreads = 128;
constexpr int kMuRows = 256;       // mu_psi rows staged in shared memory at a time
constexpr int kWienerChunk = 64;   // Wiener denominators per thread (sliding window)
constexpr int64_t kTargetThreads = 152 * 4096;   // correlation threads aimed for (chunks S)

inline size_t align_up(size_t x) { return (x + 255) / 256 * 256; }

template <class T>
T* at(void* ws, size_t off) {
    return reinterpret_cast<T*>(static_cast<char*>(ws) + off);
}

struct NlsaLayout {
    int64_t K = 0;              // elements per image in the correlation (spectrum or pixels)
    int S = 1, chunk = 0, groups = 1;
    bool smem_fft = false;
    size_t twid = 0, spec = 0, rw = 0, mu = 0, part = 0, G = 0, img = 0, work = 0, total = 0;
    size_t work_bytes = 0;
};

NlsaLayout nlsa_layout(int N, int num, int c, int T, bool wiener) {
    NlsaLayout L;
    const int m = num - c;
    const int Nh = N / 2 + 1;
    const int64_t NN = (int64_t)N * N;
    L.K = wiener ? (int64_t)N * Nh : NN;
    L.groups = (T + kModes - 1) / kModes;
    const int64_t lag_blocks = (c + kLags - 1) / kLags;
    int64_t S = (kTargetThreads + L.K * lag_blocks - 1) / (L.K * lag_blocks);
    S = std::max<int64_t>(1, std::min<int64_t>({S, 64, (int64_t)m}));
    L.chunk = (int)((m + S - 1) / S);
    L.S = (m + L.chunk - 1) / L.chunk;
    L.smem_fft = wiener && (N == 32 || N == 64 || N == 128);
    const size_t vsz = wiener ? sizeof(float2) : sizeof(float);
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off += align_up(bytes);
        return o;
    };
    L.part = take(vsz * (size_t)L.S * c * kModes * L.K);
    L.mu = take(sizeof(float) * (size_t)L.groups * m * kModes);
    if (wiener) {
        L.twid = take(sizeof(float2) * Nh);
        L.spec = take(sizeof(float2) * (size_t)num * L.K);
        L.rw = take(sizeof(float) * (size_t)m * L.K);
        L.G = take(sizeof(float2) * (size_t)c * kModes * L.K);
        L.img = take(sizeof(float) * (size_t)c * kModes * NN);
        if (!L.smem_fft) {
            L.work_bytes = 2 * std::max(fft_work_bytes(N, CUFFT_R2C, num),
                                        fft_work_bytes(N, CUFFT_C2R, (int64_t)c * kModes));
            L.work = take(L.work_bytes);
        }
    }
    L.total = off;
    return L;
}

__global__ void con_distances_kernel(const double* __restrict__ DD, int num, int c, int m,
                                     double* __restrict__ out) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= m) return;
    for (int a = blockIdx.y; a < m; a += gridDim.y) {
        const double* p = DD + (int64_t)a * num + b;
        double s = 0.0;
        for (int i = 0; i < c; ++i) s += p[(int64_t)i * (num + 1)];
        out[(int64_t)a * m + b] = s;
    }
}

// exp(-2 pi i k / N), k = 0..N/2, evaluated in double
__global__ void twiddle_kernel(int N, float2* __restrict__ tw) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k > N / 2) return;
    double sn, cs;
    sincospi(-2.0 * k / N, &sn, &cs);
    tw[k] = make_float2((float)cs, (float)sn);
}

// rw[i][k] = 1 / wd_i(k), wd_i = sum_{t = i+1 .. i+c} C_t(k)^2 + 1/5 (get_wiener.py:14-19), C_t(k)
// = ctf[t][ky][kx] for half-plane frequency k = ky Nh + kx.  Each thread starts its chunk of i
// with the direct sum (t = i+c first, as the reference adds) and slides it in float64; the
// reciprocal is taken in float32 (the correlation's precision).
__global__ void wiener_kernel(const float* __restrict__ ctf, int N, int Nh, int64_t K, int c,
                              int m, float* __restrict__ rw) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= K) return;
    const int ky = (int)(k / Nh);
    const int kx = (int)(k - (int64_t)ky * Nh);
    const int64_t NN = (int64_t)N * N;
    const float* C = ctf + (int64_t)ky * N + kx;
    const int i0 = blockIdx.y * kWienerChunk;
    const int i1 = min(m, i0 + kWienerChunk);
    double w = 0.0;
    for (int t = i0 + c; t > i0; --t) {
        const double v = C[t * NN];
        w += v * v;
    }
    for (int i = i0; i < i1; ++i) {
        rw[(int64_t)i * K + k] = __frcp_rn((float)(w + 0.2));
        if (i + 1 < i1) {
            const double a = C[(int64_t)(i + 1 + c) * NN], b = C[(int64_t)(i + 1) * NN];
            w += a * a - b * b;
        }
    }
}

// mu[g][i][l] = mu_psi[i][kModes g + l] in float32, zero past the last mode
__global__ void mu_kernel(const double* __restrict__ mu_psi, int m, int T, int groups,
                          float* __restrict__ mu) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= (int64_t)groups * m * kModes) return;
    const int l = (int)(e % kModes);
    const int64_t i = (e / kModes) % m;
    const int g = (int)(e / ((int64_t)m * kModes));
    const int col = g * kModes + l;
    mu[e] = col < T ? (float)mu_psi[i * T + col] : 0.f;
}

__device__ __forceinline__ float2 vscale(float2 v, float s) { return make_float2(v.x * s, v.y * s); }
__device__ __forceinline__ float vscale(float v, float s) { return v * s; }
__device__ __forceinline__ float2 vfma(float2 a, float g, float2 acc) {
    return __ffma2_rn(a, make_float2(g, g), acc);
}
__device__ __forceinline__ float vfma(float a, float g, float acc) { return fmaf(a, g, acc); }
template <class V> __device__ __forceinline__ V vzero();
template <> __device__ __forceinline__ float2 vzero<float2>() { return make_float2(0.f, 0.f); }
template <> __device__ __forceinline__ float vzero<float>() { return 0.f; }

// part[s][ii][l][k] = sum_{i in chunk s} h_{i+c-1-ii}(k) w_i(k) mu[i][l]; h_j = data[j][k]
// (times ctf[j] at k when WEIGHTED), w_i = rw[i][k] (WEIGHTED) or 1
template <class V, bool WEIGHTED>
__global__ void __launch_bounds__(kCorrThreads) correlate_kernel(
        const V* __restrict__ data, const float* __restrict__ ctf, const float* __restrict__ rw,
        const float* __restrict__ mu, int64_t K, int N, int Nh, int num, int c, int m,
        int chunk, V* __restrict__ part) {
    __shared__ float4 mus[kMuRows][2];
    const int64_t k = blockIdx.x * (int64_t)kCorrThreads + threadIdx.x;
    const bool valid = k < K;
    const int64_t kk = valid ? k : 0;
    const int ii0 = blockIdx.y * kLags;
    const int i0 = blockIdx.z * chunk;
    const int i1 = min(m, i0 + chunk);
    int64_t coff = 0;
    if (WEIGHTED) {
        const int ky = (int)(kk / Nh);
        coff = (int64_t)ky * N + (kk - (int64_t)ky * Nh);
    }
    const int64_t NN = (int64_t)N * N;
    auto load = [&](int j) -> V {
        j = min(max(j, 0), num - 1);
        V v = data[(int64_t)j * K + kk];
        if (WEIGHTED) v = vscale(v, ctf[(int64_t)j * NN + coff]);
        return v;
    };
    V win[kLags];
#pragma unroll
    for (int b = 0; b < kLags; ++b) win[b] = load(i0 + c - 1 - ii0 - b);
    V acc[kLags][kModes];
#pragma unroll
    for (int b = 0; b < kLags; ++b)
#pragma unroll
        for (int l = 0; l < kModes; ++l) acc[b][l] = vzero<V>();
    float w_next = WEIGHTED && i0 < i1 ? rw[(int64_t)i0 * K + kk] : 1.f;
    for (int base = i0; base < i1; base += kMuRows) {
        const int n = min(kMuRows, i1 - base);
        __syncthreads();
        for (int e = threadIdx.x; e < 2 * n; e += kCorrThreads)
            mus[e >> 1][e & 1] =
                    reinterpret_cast<const float4*>(mu + (int64_t)(base + (e >> 1)) * kModes)[e & 1];
        __syncthreads();
        for (int t = 0; t < n; ++t) {
            const int i = base + t;
            const float w = w_next;
            const V nxt = load(i + c - ii0);                  // window head of step i + 1
            if (WEIGHTED && i + 1 < i1) w_next = rw[(int64_t)(i + 1) * K + kk];
            const float4 m0 = mus[t][0], m1 = mus[t][1];
            const float g[kModes] = {w * m0.x, w * m0.y, w * m0.z, w * m0.w,
                                     w * m1.x, w * m1.y, w * m1.z, w * m1.w};
#pragma unroll
            for (int b = 0; b < kLags; ++b)
#pragma unroll
                for (int l = 0; l < kModes; ++l) acc[b][l] = vfma(win[b], g[l], acc[b][l]);
#pragma unroll
            for (int b = kLags - 1; b > 0; --b) win[b] = win[b - 1];
            win[0] = nxt;
        }
    }
    if (!valid) return;
#pragma unroll
    for (int b = 0; b < kLags; ++b) {
        const int ii = ii0 + b;
        if (ii >= c) break;
#pragma unroll
        for (int l = 0; l < kModes; ++l)
            part[(((int64_t)blockIdx.z * c + ii) * kModes + l) * K + k] = acc[b][l];
    }
}

// G[q][k] = sum_s part[s][q][k] in a fixed order (q = ii kModes + l)
__global__ void reduce_parts_kernel(const float2* __restrict__ part, int S, int64_t total,
                                    float2* __restrict__ G) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= total) return;
    double re = 0.0, im = 0.0;
    for (int s = 0; s < S; ++s) {
        const float2 v = part[(int64_t)s * total + e];
        re += v.x;
        im += v.y;
    }
    G[e] = make_float2((float)re, (float)im);
}

// A[(ii NN + x N + y) T + l0 + l] = msk[y][x] * scale * img[ii kModes + l][y][x], l < nl: the
// snapshot transposed and flattened (NLSA.py:80); y runs fastest over the threads
__global__ void scatter_kernel(const float* __restrict__ img, const double* __restrict__ msk,
                               double scale, int N, int c, int T, int l0, int nl,
                               double* __restrict__ A) {
    const int64_t NN = (int64_t)N * N;
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= (int64_t)c * NN) return;
    const int ii = (int)(e / NN);
    const int64_t p = e - (int64_t)ii * NN;          // p = x N + y
    const int x = (int)(p / N), y = (int)(p - (int64_t)x * N);
    const double f = msk ? msk[(int64_t)y * N + x] * scale : scale;
    double* dst = A + ((int64_t)ii * NN + p) * T + l0;
    for (int l = 0; l < nl; ++l)
        dst[l] = f * (double)img[((int64_t)ii * kModes + l) * NN + (int64_t)y * N + x];
}

// unfiltered branch: A[(ii NN + x N + y) T + l0 + l] = sum_s part[s][ii][l][y N + x]
__global__ void reduce_scatter_kernel(const float* __restrict__ part, int S, int N, int c, int T,
                                      int l0, int nl, double* __restrict__ A) {
    const int64_t NN = (int64_t)N * N;
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= (int64_t)c * NN) return;
    const int ii = (int)(e / NN);
    const int64_t p = e - (int64_t)ii * NN;
    const int x = (int)(p / N), y = (int)(p - (int64_t)x * N);
    const int64_t total = (int64_t)c * kModes * NN;
    double* dst = A + ((int64_t)ii * NN + p) * T + l0;
    for (int l = 0; l < nl; ++l) {
        const int64_t q = ((int64_t)ii * kModes + l) * NN + (int64_t)y * N + x;
        double s = 0.0;
        for (int t = 0; t < S; ++t) s += part[(int64_t)t * total + q];
        dst[l] = s;
    }
}

unsigned blocks_for(int64_t n, int threads) { return (unsigned)((n + threads - 1) / threads); }

}  // namespace
}  // namespace mem

using namespace mem;

extern "C" {

int mem_nlsa_con_distances(const double* DD, int32_t num, int32_t c, double* ConD,
                           void* stream) {
    if (!DD || !ConD || num < 2 || c < 1 || c >= num) return MEM_ERR_INVALID;
    const int m = num - c;
    dim3 grid(blocks_for(m, 128), (unsigned)std::min(m, 65535));
    con_distances_kernel<<<grid, 128, 0, (cudaStream_t)stream>>>(DD, num, c, m, ConD);
    MEM_LAUNCH_CHECK();
    return MEM_OK;
}

int mem_nlsa_workspace_size(int32_t N, int32_t num, int32_t c, int32_t n_modes, int32_t wiener,
                            size_t* bytes) {
    if (!bytes || N < 2 || N > kMaxN || num < 2 || c < 1 || c >= num || n_modes < 1 ||
        n_modes > 64)
        return MEM_ERR_INVALID;
    *bytes = nlsa_layout(N, num, c, n_modes, wiener != 0).total;
    return MEM_OK;
}

int mem_nlsa_snapshots(int32_t N, int32_t num, int32_t c, int32_t n_modes, const float* images,
                       const float* ctf, const double* mu_psi, const double* msk2,
                       void* workspace, size_t workspace_bytes, double* A, void* stream) {
    if (!images || !mu_psi || !A || N < 2 || N > kMaxN || num < 2 || c < 1 || c >= num ||
        n_modes < 1 || n_modes > 64)
        return MEM_ERR_INVALID;
    const bool wiener = ctf != nullptr;
    const NlsaLayout L = nlsa_layout(N, num, c, n_modes, wiener);
    if (!workspace || workspace_bytes < L.total) return MEM_ERR_WORKSPACE;
    cudaStream_t s = (cudaStream_t)stream;
    const int m = num - c;
    const int Nh = N / 2 + 1;
    const int64_t NN = (int64_t)N * N;
    float* mu = at<float>(workspace, L.mu);
    mu_kernel<<<blocks_for((int64_t)L.groups * m * kModes, 256), 256, 0, s>>>(
            mu_psi, m, n_modes, L.groups, mu);
    MEM_LAUNCH_CHECK();
    const dim3 cgrid(blocks_for(L.K, kCorrThreads), (unsigned)((c + kLags - 1) / kLags),
                     (unsigned)L.S);
    if (!wiener) {
        float* part = at<float>(workspace, L.part);
        for (int g = 0; g < L.groups; ++g) {
            correlate_kernel<float, false><<<cgrid, kCorrThreads, 0, s>>>(
                    images, nullptr, nullptr, mu + (int64_t)g * m * kModes, L.K, N, Nh, num, c,
                    m, L.chunk, part);
            MEM_LAUNCH_CHECK();
            const int nl = std::min(kModes, n_modes - g * kModes);
            reduce_scatter_kernel<<<blocks_for((int64_t)c * NN, 256), 256, 0, s>>>(
                    part, L.S, N, c, n_modes, g * kModes, nl, A);
            MEM_LAUNCH_CHECK();
        }
        return MEM_OK;
    }
    // Wiener branch: half-plane spectra of the images, denominators, correlation per mode group,
    // inverse transforms of the c x kModes sums, scatter
    mem_plan fp;
    fp.N = N;
    fp.Nh = Nh;
    MEM_CUDA_TRY(cudaGetDevice(&fp.device));
    float2* twid = at<float2>(workspace, L.twid);
    float2* spec = at<float2>(workspace, L.spec);
    float* rw = at<float>(workspace, L.rw);
    float2* G = at<float2>(workspace, L.G);
    float* img = at<float>(workspace, L.img);
    void* work = L.work_bytes ? at<char>(workspace, L.work) : nullptr;
    if (L.smem_fft) {
        twiddle_kernel<<<1, 256, 0, s>>>(N, twid);
        MEM_LAUNCH_CHECK();
        int st = kern::spectrum_fft(fp, num, images, twid, spec, s);
        if (st != MEM_OK) return st;
    } else {
        int st = fft_exec(fp.device, N, CUFFT_R2C, num, NN, L.K, const_cast<float*>(images), spec,
                          work, s);
        if (st != MEM_OK) return st;
    }
    wiener_kernel<<<dim3(blocks_for(L.K, 128), blocks_for(m, kWienerChunk)), 128, 0, s>>>(
            ctf, N, Nh, L.K, c, m, rw);
    MEM_LAUNCH_CHECK();
    float2* part = at<float2>(workspace, L.part);
    const int64_t total = (int64_t)c * kModes * L.K;
    for (int g = 0; g < L.groups; ++g) {
        correlate_kernel<float2, true><<<cgrid, kCorrThreads, 0, s>>>(
                spec, ctf, rw, mu + (int64_t)g * m * kModes, L.K, N, Nh, num, c, m, L.chunk,
                part);
        MEM_LAUNCH_CHECK();
        reduce_parts_kernel<<<blocks_for(total, 256), 256, 0, s>>>(part, L.S, total, G);
        MEM_LAUNCH_CHECK();
        int st = L.smem_fft
                ? kern::inverse_fft(fp, (int64_t)c * kModes, G, twid, img, nullptr, false, s)
                : fft_exec(fp.device, N, CUFFT_C2R, (int64_t)c * kModes, L.K, NN, G, img, work,
                           s);
        if (st != MEM_OK) return st;
        const int nl = std::min(kModes, n_modes - g * kModes);
        scatter_kernel<<<blocks_for((int64_t)c * NN, 256), 256, 0, s>>>(
                img, msk2, 1.0 / (double)NN, N, c, n_modes, g * kModes, nl, A);
        MEM_LAUNCH_CHECK();
    }
    return MEM_OK;
}

}  // extern "C"
