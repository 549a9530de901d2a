// Diffusion-map embedding of one PD's distance matrix on the GPU: the dense-matrix work of
// DMembeddingII.op (reference modules/DMembeddingII.py:86-185) with fergusonE.op
// (modules/fergusonE.py:33-58) and slaplacianonFly.op (modules/slaplacianonFly.py:42-81).
//
//   1. symmetrised squared distances (DMembeddingII.py:112-139, construct_matrix0/1 :72-84):
//        s_ij = sqrt(D_ji) if j is among the k nearest of point i (column i of D, the point itself
//               first), D_ji >= 1e-6 and j != i; else 0
//        Y_ij = s_ij^2 + s_ji^2 - s_ij s_ji
//      entry (i, j) is an edge if Y_ij != 0 or if j is a listed neighbour of i with D_ji < 1e-6
//      (or j = i); non-edges are stored as -1;
//   2. bandwidth sweep (fergusonE.py:36-44): for every log eps,
//        sum over edges of exp(-Y/(2 eps)) for the terms with Y/(2 eps) < thr;
//   3. normalised kernel (slaplacianonFly.py:55-80, alpha = 1):
//        W = exp(-Y/sigma^2) on edges; W'_ij = W_ij/(d_i d_j), d = column sums of W;
//        L_ij = W'_ij/(e_i e_j), e = sqrt(column sums of W'); L = |L + L^T|/2.
// The eigen-decomposition of L, the tanh fit of the sweep and the neighbour lists (a sort per
// column) stay with the caller.  The sweep evaluates exp in float32 and sums in float64 per
// block; everything else is float64.
#include <cstdint>

#include "mem_internal.cuh"

namespace mem {
namespace {

constexpr double kZeroDist = 1e-6;
constexpr int kTile = 32;

// 1. Y from D (row-major n x n); listed = nullptr: every entry is a listed neighbour (k = n)
__global__ void dm_sym_kernel(const double* __restrict__ D, int64_t n,
                              const uint8_t* __restrict__ listed, double* __restrict__ Y) {
    __shared__ double tD[kTile][kTile + 1];      // D block transposed: the (j, i) entries
    __shared__ uint8_t tL[kTile][kTile + 1];
    const int64_t bi = (int64_t)blockIdx.y * kTile, bj = (int64_t)blockIdx.x * kTile;
    const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8 threads
    for (int r = ty; r < kTile; r += 8) {
        const int64_t gi = bj + r, gj = bi + tx;   // load D[bj + r][bi + tx]
        const bool in = gi < n && gj < n;
        tD[tx][r] = in ? D[gi * n + gj] : 0.0;
        tL[tx][r] = in ? (listed ? listed[gi * n + gj] : (uint8_t)1) : (uint8_t)0;
    }
    __syncthreads();
    for (int r = ty; r < kTile; r += 8) {
        const int64_t i = bi + r, j = bj + tx;
        if (i >= n || j >= n) continue;
        const double dij = D[i * n + j];           // D_ij: value of s_ji
        const double dji = tD[r][tx];              // D_ji: value of s_ij
        const bool lij = listed ? listed[i * n + j] != 0 : true;   // j listed for point i
        const bool lji = tL[r][tx] != 0;                              // i listed for point j
        const double sij = (lij && i != j && dji >= kZeroDist) ? sqrt(dji) : 0.0;
        const double sji = (lji && i != j && dij >= kZeroDist) ? sqrt(dij) : 0.0;
        const double y = sij * sij + sji * sji - sij * sji;
        const bool zero_edge = lij && (i == j || dji < kZeroDist);
        Y[i * n + j] = (y != 0.0 || zero_edge) ? y : -1.0;
    }
}

// 2. sweep partial sums; every thread holds kPer entries of Y and walks all the log eps values
constexpr int kSweepThreads = 256, kPer = 8, kMaxEps = 2048;

__global__ void __launch_bounds__(kSweepThreads) dm_sweep_kernel(
        const double* __restrict__ Y, int64_t total, const float* __restrict__ scale,
        int n_eps, float thr, double* __restrict__ sums) {
    __shared__ double part[kMaxEps];
    for (int e = threadIdx.x; e < n_eps; e += kSweepThreads) part[e] = 0.0;
    float y[kPer];
    const int64_t base = ((int64_t)blockIdx.x * kSweepThreads + threadIdx.x) * kPer;
#pragma unroll
    for (int u = 0; u < kPer; ++u) {
        const int64_t g = base + u;
        y[u] = g < total ? (float)Y[g] : -1.0f;     // -1: not an edge
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    for (int e = 0; e < n_eps; ++e) {
        const float c = scale[e];                   // log2(e) / (2 eps)
        const float tl = thr * 1.4426950408889634f; // the threshold on d = Y/(2 eps), base 2
        float acc = 0.f;
#pragma unroll
        for (int u = 0; u < kPer; ++u) {
            // d log2(e); scale is +inf for the smallest eps (beyond float range): zero-distance
            // edges still give exp(0) = 1 there, all others are beyond the threshold
            const float d2 = y[u] == 0.f ? 0.f : y[u] * c;
            acc += (y[u] >= 0.f && d2 < tl) ? exp2f(-d2) : 0.f;
        }
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0 && acc != 0.f) atomicAdd(&part[e], (double)acc);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < n_eps; e += kSweepThreads)
        if (part[e] != 0.0) atomicAdd(&sums[e], part[e]);
}

// 3a. W = exp(-Y / sigma^2) on edges (in place over Y) and its column sums
__global__ void dm_weights_kernel(double* __restrict__ W, int64_t n, double inv_s2,
                                  double* __restrict__ colsum) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    double s = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        const double y = W[i * n + j];
        const double w = y >= 0.0 ? exp(-y * inv_s2) : 0.0;
        W[i * n + j] = w;
        s += w;
    }
    colsum[j] = s;
}

// 3b. W'_ij = W_ij / (d_i d_j) in place, and e_j = sqrt(column sums of W')
__global__ void dm_normalise_kernel(double* __restrict__ W, int64_t n,
                                    const double* __restrict__ d, double* __restrict__ e) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const double dj = d[j];
    double s = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        const double w = W[i * n + j] / (d[i] * dj);
        W[i * n + j] = w;
        s += w;
    }
    e[j] = sqrt(s);
}

// 3c. L_ij = W'_ij / (e_i e_j), then L = |L + L^T| / 2 (tile pairs (bi, bj), (bj, bi))
__global__ void dm_finish_kernel(double* __restrict__ W, int64_t n, const double* __restrict__ e) {
    __shared__ double ta[kTile][kTile + 1], tb[kTile][kTile + 1];
    const int64_t bi = (int64_t)blockIdx.y * kTile, bj = (int64_t)blockIdx.x * kTile;
    if (bj < bi) return;                           // each unordered tile pair once
    const int tx = threadIdx.x, ty = threadIdx.y;
    for (int r = ty; r < kTile; r += 8) {
        const int64_t i = bi + r, j = bj + tx;
        ta[r][tx] = (i < n && j < n) ? W[i * n + j] / (e[i] * e[j]) : 0.0;
        const int64_t i2 = bj + r, j2 = bi + tx;
        tb[r][tx] = (i2 < n && j2 < n) ? W[i2 * n + j2] / (e[i2] * e[j2]) : 0.0;
    }
    __syncthreads();
    for (int r = ty; r < kTile; r += 8) {
        const int64_t i = bi + r, j = bj + tx;
        if (i < n && j < n) W[i * n + j] = fabs(ta[r][tx] + tb[tx][r]) / 2.0;
        const int64_t i2 = bj + r, j2 = bi + tx;
        if (i2 < n && j2 < n) W[i2 * n + j2] = fabs(tb[r][tx] + ta[tx][r]) / 2.0;
    }
}

}  // namespace
}  // namespace mem

using namespace mem;

extern "C" {

int mem_dm_symmetrise(const double* D, int64_t n, const uint8_t* listed, double* Y,
                      void* stream) {
    if (!D || !Y || n < 1) return MEM_ERR_INVALID;
    const unsigned nb = (unsigned)((n + kTile - 1) / kTile);
    dm_sym_kernel<<<dim3(nb, nb), dim3(kTile, 8), 0, (cudaStream_t)stream>>>(D, n, listed, Y);
    MEM_LAUNCH_CHECK();
    return MEM_OK;
}

int mem_dm_sweep(const double* Y, int64_t n, const float* scale, int32_t n_eps, double thr,
                 double* sums, void* stream) {
    if (!Y || !scale || !sums || n < 1 || n_eps < 1 || n_eps > kMaxEps) return MEM_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    MEM_CUDA_TRY(cudaMemsetAsync(sums, 0, sizeof(double) * n_eps, s));
    const int64_t total = n * n;
    const int64_t per_block = (int64_t)kSweepThreads * kPer;
    dm_sweep_kernel<<<(unsigned)((total + per_block - 1) / per_block), kSweepThreads, 0, s>>>(
            Y, total, scale, n_eps, (float)thr, sums);
    MEM_LAUNCH_CHECK();
    return MEM_OK;
}

int mem_dm_laplacian(double* Y, int64_t n, double sigma, double* scratch, void* stream) {
    if (!Y || !scratch || n < 1 || !(sigma > 0.0)) return MEM_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    const unsigned nb1 = (unsigned)((n + 127) / 128);
    dm_weights_kernel<<<nb1, 128, 0, s>>>(Y, n, 1.0 / (sigma * sigma), scratch);
    MEM_LAUNCH_CHECK();
    dm_normalise_kernel<<<nb1, 128, 0, s>>>(Y, n, scratch, scratch + n);
    MEM_LAUNCH_CHECK();
    const unsigned nb = (unsigned)((n + kTile - 1) / kTile);
    dm_finish_kernel<<<dim3(nb, nb), dim3(kTile, 8), 0, s>>>(Y, n, scratch + n);
    MEM_LAUNCH_CHECK();
    return MEM_OK;
}

}  // extern "C"
