// RELION branch of the image read (reference modules/getDistanceCTF_local_Conj9combinedS2.py
// :259-264): the particle image as stored in the MRC stack (no transpose), shifted by
// (sh_y - 0.5, sh_x - 0.5) with scipy.ndimage.shift(order=3, mode='wrap').
//
// That scipy call (measured against scipy 1.18 to 1e-15) is a cubic B-spline shift whose
//   * coefficients come from the mirror-boundary prefilter (the 'mirror' spline filter: the
//     signal extended symmetrically, period 2N-2) along each axis;
//   * sample coordinate u = i - s is wrapped with period N-1 into [0, N-1] when it falls outside;
//   * four taps floor(u)-1 .. floor(u)+2 take mirrored indices (k -> -k, N-1+k -> N-1-k).
// A shift has one fractional offset per axis, so the 2D interpolation is two separable 4-tap
// passes.  The mirror prefilter uses the closed-form start values of the causal and anticausal
// recursions (exact for the symmetric extension).
//
// Output: the shifted image transposed (out[a][b] = I[b][a]), i.e. laid out as a SPIDER stack
// image is, so the rest of the stage (conjugate flip, normalisation, low-pass, ...) reads it
// unchanged.  One CTA per image, the image in shared memory (row stride N + 1), N <= 236.
#include <cmath>

#include "mem_internal.cuh"

namespace mem {
namespace {

constexpr float kPole = -0.26794919243112270f;   // sqrt(3) - 2

__device__ __forceinline__ int mirror_index(int k, int N) {
    const int P = 2 * N - 2;
    if (P <= 0) return 0;
    k %= P;
    if (k < 0) k += P;
    return k >= N ? P - k : k;
}

// mirror-boundary cubic B-spline prefilter of one line x[0..N-1] (stride st) in place
__device__ void mirror_prefilter_line(float* x, int N, int st) {
    if (N < 2) return;
    const float z = kPole;
    // causal start: sum over one period of the symmetric extension, / (1 - z^(2N-2))
    float zk = z, s = x[0];
    const int L = 2 * N - 2;
    float zL = 1.f;
    for (int k = 0; k < L; ++k) zL *= z;
    float zLk = zL / z;                     // z^(L-1)
    for (int k = 1; k < N - 1; ++k) {
        s += (zk + zLk) * x[k * st];
        zk *= z;
        zLk /= z;
    }
    s += zk * x[(N - 1) * st];              // z^(N-1) x[N-1]
    float cp = s / (1.f - zL);
    x[0] = cp;
    for (int k = 1; k < N; ++k) {
        cp = x[k * st] + z * cp;
        x[k * st] = cp;
    }
    // anticausal start for the mirror boundary, then c-[k] = z (c-[k+1] - c+[k]); output 6 c-
    float cm = (z / (z * z - 1.f)) * (x[(N - 1) * st] + z * x[(N - 2) * st]);
    x[(N - 1) * st] = 6.f * cm;
    for (int k = N - 2; k >= 0; --k) {
        cm = z * (cm - x[k * st]);
        x[k * st] = 6.f * cm;
    }
}

__device__ __forceinline__ void bspline4(float t, float w[4]) {
    const float u = 1.0f - t;
    const float t2 = t * t, u2 = u * u;
    w[0] = (1.0f / 6.0f) * u2 * u;
    w[3] = (1.0f / 6.0f) * t2 * t;
    w[1] = (2.0f / 3.0f) - t2 * (1.0f - 0.5f * t);
    w[2] = (2.0f / 3.0f) - u2 * (1.0f - 0.5f * u);
}

// the wrapped sample coordinate of output index i for shift s: first tap and fraction
__device__ __forceinline__ void wrap_coord(int i, double s, int N, int* f, float* t) {
    double u = (double)i - s;
    const double per = (double)(N - 1);
    if (per > 0.0 && (u < 0.0 || u > per)) u -= per * floor(u / per);
    const double fu = floor(u);
    *f = (int)fu;
    *t = (float)(u - fu);
}

constexpr int kMaxPer = 8;                         // N <= 256: outputs per lane and line

// Interpolation along one axis, one warp per line, in place: lane l computes the outputs
// j = l + 32 q of its line into registers, then writes them (taps and weights per j are the
// same for every line and are computed once).  Lines are rows (axis 1, stride 1 along the line)
// or columns (axis 0, stride P).
__device__ __forceinline__ void shift_lines(float* A, int N, int P, double sh, int line_stride,
                                            int elem_stride, int nwarps) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int tap[kMaxPer][4];
    float w[kMaxPer][4];
#pragma unroll
    for (int q = 0; q < kMaxPer; ++q) {
        const int j = lane + 32 * q;
        int f = 0;
        float t = 0.f;
        if (j < N) wrap_coord(j, sh, N, &f, &t);
        bspline4(t, w[q]);
#pragma unroll
        for (int b = 0; b < 4; ++b) tap[q][b] = mirror_index(f - 1 + b, N) * elem_stride;
    }
    for (int line = warp; line < N; line += nwarps) {
        float* x = A + line * line_stride;
        float v[kMaxPer];
#pragma unroll
        for (int q = 0; q < kMaxPer; ++q) {
            float acc = 0.f;
            if (lane + 32 * q < N) {
#pragma unroll
                for (int b = 0; b < 4; ++b) acc = fmaf(w[q][b], x[tap[q][b]], acc);
            }
            v[q] = acc;
        }
        __syncwarp();
#pragma unroll
        for (int q = 0; q < kMaxPer; ++q)
            if (lane + 32 * q < N) x[(lane + 32 * q) * elem_stride] = v[q];
        __syncwarp();
    }
}

template <int NT>
__global__ void __launch_bounds__(NT) relion_shift_kernel(
        const float* __restrict__ stack, int64_t num_stack, const int64_t* __restrict__ sidx,
        const double* __restrict__ shift_yx, int N, float* __restrict__ out,
        uint32_t* __restrict__ status) {
    extern __shared__ float A[];           // the image, [N][N+1]
    const int P = N + 1;
    const int64_t img = blockIdx.x;
    const int64_t s = sidx[img];
    float* dst = out + img * (int64_t)N * N;
    const int NN = N * N;
    if (s < 0 || s >= num_stack) {
        if (threadIdx.x == 0) atomicOr(status, 2u);
        for (int p = threadIdx.x; p < NN; p += NT) dst[p] = __int_as_float(0x7fc00000);
        return;
    }
    const float* src = stack + s * (int64_t)NN;
    for (int p = threadIdx.x; p < NN; p += NT) {
        const int r = p / N, c = p - r * N;
        A[r * P + c] = src[p];
    }
    __syncthreads();
    for (int r = threadIdx.x; r < N; r += NT) mirror_prefilter_line(A + r * P, N, 1);   // axis 1
    __syncthreads();
    for (int c = threadIdx.x; c < N; c += NT) mirror_prefilter_line(A + c, N, P);       // axis 0
    __syncthreads();
    // axis 1 (shift sh_x - 0.5), then axis 0 (shift sh_y - 0.5)
    shift_lines(A, N, P, shift_yx[2 * img + 1], P, 1, NT / 32);
    __syncthreads();
    shift_lines(A, N, P, shift_yx[2 * img], 1, P, NT / 32);
    __syncthreads();
    // transposed store: out[a][b] = I[b][a]
    for (int p = threadIdx.x; p < NN; p += NT) {
        const int a = p / N, b = p - a * N;
        dst[p] = A[b * P + a];
    }
}

}  // namespace

namespace kern {
int relion_shift(const mem_plan& P, const mem_inputs& in, float* out, uint32_t* status,
                 cudaStream_t s) {
    if (P.n_images == 0) return MEM_OK;
    const int N = P.N;
    if (N > kMaxSmemN) return MEM_ERR_UNSUPPORTED;         // one image in shared memory
    const size_t smem = (size_t)N * (N + 1) * sizeof(float);
    constexpr int NT = 256;
    MEM_CUDA_TRY(cudaFuncSetAttribute(relion_shift_kernel<NT>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    relion_shift_kernel<NT><<<(unsigned)P.n_images, NT, smem, s>>>(
            in.stack, in.num_stack, in.stack_index, in.shift_yx, N, out, status);
    MEM_LAUNCH_CHECK();
    return MEM_OK;
}
}  // namespace kern
}  // namespace mem
