// Volume mask of the distance stage (reference modules/getDistanceCTF_local_Conj9combinedS2.py
// :303-310, projectMask.op modules/projectMask.py:118-135): the mask volume rotated to the PD's
// direction with scipy.ndimage.affine_transform (order 3, mode 'nearest'), summed along z and
// thresholded at 1 gives the 2D mask msk2 that multiplies every rotated image before its
// spectrum (:344) -- and through the spectra the averages (:366-367).
//
// In the scipy here (1.18) an order-3 'nearest' interpolation is (measured to 3e-15 against
// affine_transform on 3D volumes): the volume padded by 12 samples per side with its edge
// values, the 'reflect' spline prefilter of the padded volume along each axis, then the
// tensor-product cubic B-spline with tap indices clamped to the padded volume.  The 'reflect'
// prefilter of a line is the exact periodic prefilter of its half-sample-symmetric extension
// (period 2M).  Everything here is float64: the mask is a threshold of a sum.
#include <cmath>

#include "mem_internal.cuh"

namespace mem {
namespace {

constexpr int kMaskPad = 12;
constexpr int kMaxM = kMaxSmemN + 2 * kMaskPad;
constexpr double kPoleD = -0.2679491924311227065;   // sqrt(3) - 2

// P[a][b][c] (M^3, M = N + 24) = swapaxes(vol, 0, 2) padded with edge values; vol is (N, N, N)
// as stored (z, y, x), so P[a][b][c] = vol[cc][cb][ca] with (ca, cb, cc) the clamped indices
__global__ void mask_pad_kernel(const float* __restrict__ vol, int N, double* __restrict__ P) {
    const int M = N + 2 * kMaskPad;
    const int64_t total = (int64_t)M * M * M;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int a = (int)(e / ((int64_t)M * M));
        const int b = (int)((e / M) % M), c = (int)(e % M);
        const int ca = min(max(a - kMaskPad, 0), N - 1);
        const int cb = min(max(b - kMaskPad, 0), N - 1);
        const int cc = min(max(c - kMaskPad, 0), N - 1);
        P[e] = (double)vol[((int64_t)cc * N + cb) * N + ca];
    }
}

// 'reflect' cubic B-spline prefilter along one axis of P, one thread per line
__global__ void mask_prefilter_kernel(double* __restrict__ P, int M, int axis) {
    const int64_t line = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (line >= (int64_t)M * M) return;
    const int64_t u = line / M, v = line % M;
    int64_t base, st;
    if (axis == 0) { base = u * M + v; st = (int64_t)M * M; }
    else if (axis == 1) { base = u * M * M + v; st = M; }
    else { base = (u * M + v) * M; st = 1; }
    const int L = 2 * M;
    double y[2 * kMaxM];
    for (int k = 0; k < M; ++k) {
        const double x = P[base + k * st];
        y[k] = x;
        y[L - 1 - k] = x;
    }
    const double z = kPoleD;
    double zL = 1.0;
    for (int k = 0; k < L; ++k) zL *= z;
    // causal: start value = sum_k z^k y[-k mod L] / (1 - z^L)
    double s = y[0], zk = z;
    for (int k = 1; k < L; ++k) {
        s += zk * y[L - k];
        zk *= z;
    }
    y[0] = s / (1.0 - zL);
    for (int k = 1; k < L; ++k) y[k] += z * y[k - 1];
    // anticausal d[k] = c+[k] + z d[k+1], start value sum_j z^j c+[(L-1+j) mod L] / (1 - z^L)
    double t = y[L - 1];
    zk = z;
    for (int j = 1; j < L; ++j) {
        t += zk * y[j - 1];
        zk *= z;
    }
    double d = t / (1.0 - zL);
    y[L - 1] = d;
    for (int k = L - 2; k >= 0; --k) {
        d = y[k] + z * d;
        y[k] = d;
    }
    const double gain = -6.0 * z;
    for (int k = 0; k < M; ++k) P[base + k * st] = gain * y[k];
}

__device__ __forceinline__ void bspline4d(double t, double w[4]) {
    const double u = 1.0 - t;
    const double t2 = t * t, u2 = u * u;
    w[0] = (1.0 / 6.0) * u2 * u;
    w[3] = (1.0 / 6.0) * t2 * t;
    w[1] = (2.0 / 3.0) - t2 * (1.0 - 0.5 * t);
    w[2] = (2.0 / 3.0) - u2 * (1.0 - 0.5 * u);
}

// masks[pd][a][b] = (sum_k rho(b, a, k) > 1), rho(o) = spline(C, R o + offset):
// projectMask's msk = sum(rho, axis=2).reshape(N, N).T > 1
__global__ void mask_project_kernel(const double* __restrict__ C, int N,
                                    const double* __restrict__ xf, uint8_t* __restrict__ masks) {
    const int M = N + 2 * kMaskPad;
    const int pd = blockIdx.y;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= N * N) return;
    const int i = p / N, j = p - i * N;
    const double* T = xf + 12 * pd;          // R row-major (9), offset (3)
    double sum = 0.0;
    for (int k = 0; k < N; ++k) {
        double uvw[3];
        int f[3];
        double w[3][4];
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            uvw[ax] = T[3 * ax] * i + T[3 * ax + 1] * j + T[3 * ax + 2] * k + T[9 + ax];
            const double fl = floor(uvw[ax]);
            f[ax] = (int)fl;
            bspline4d(uvw[ax] - fl, w[ax]);
        }
        double acc = 0.0;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const int64_t ia = min(max(kMaskPad + f[0] - 1 + a, 0), M - 1);
            double accb = 0.0;
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const int64_t ib = min(max(kMaskPad + f[1] - 1 + b, 0), M - 1);
                const double* row = C + (ia * M + ib) * M;
                double accc = 0.0;
#pragma unroll
                for (int c = 0; c < 4; ++c)
                    accc += w[2][c] * row[min(max(kMaskPad + f[2] - 1 + c, 0), M - 1)];
                accb += w[1][b] * accc;
            }
            acc += w[0][a] * accb;
        }
        sum += acc;
    }
    masks[(int64_t)pd * N * N + (int64_t)j * N + i] = sum > 1.0 ? 1 : 0;
}

// dst[img] = src[img] * mask of the image's PD (in place when dst == src)
__global__ void apply_pd_mask_kernel(const float* __restrict__ src, float* __restrict__ dst,
                                     const uint8_t* __restrict__ masks,
                                     const int32_t* __restrict__ img_pd, int NN) {
    const int64_t img = blockIdx.y;
    const uint8_t* m = masks + (int64_t)img_pd[img] * NN;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < NN; p += gridDim.x * blockDim.x)
        dst[img * NN + p] = m[p] ? src[img * NN + p] : 0.0f;
}

}  // namespace

namespace kern {
int apply_pd_mask(const mem_plan& P, const float* src, float* dst, const uint8_t* masks,
                  const int32_t* img_pd, cudaStream_t s) {
    if (P.n_images == 0) return MEM_OK;
    const int NN = P.N * P.N;
    dim3 grid((unsigned)std::min(64, (NN + 255) / 256), (unsigned)P.n_images);
    apply_pd_mask_kernel<<<grid, 256, 0, s>>>(src, dst, masks, img_pd, NN);
    MEM_LAUNCH_CHECK();
    return MEM_OK;
}
}  // namespace kern
}  // namespace mem

using namespace mem;

extern "C" {

int mem_mask_coefficients_size(int32_t N, size_t* bytes) {
    if (!bytes || N < 1 || N > kMaxSmemN) return MEM_ERR_INVALID;
    const size_t M = (size_t)N + 2 * kMaskPad;
    *bytes = M * M * M * sizeof(double);
    return MEM_OK;
}

int mem_mask_prepare(const float* volume, int32_t N, double* coeffs, void* stream) {
    if (!volume || !coeffs || N < 2) return MEM_ERR_INVALID;
    if (N > kMaxSmemN) return MEM_ERR_UNSUPPORTED;
    cudaStream_t s = (cudaStream_t)stream;
    const int M = N + 2 * kMaskPad;
    mask_pad_kernel<<<1024, 256, 0, s>>>(volume, N, coeffs);
    MEM_LAUNCH_CHECK();
    const unsigned nb = (unsigned)(((int64_t)M * M + 127) / 128);
    for (int axis = 0; axis < 3; ++axis) {
        mask_prefilter_kernel<<<nb, 128, 0, s>>>(coeffs, M, axis);
        MEM_LAUNCH_CHECK();
    }
    return MEM_OK;
}

int mem_mask_project(const double* coeffs, int32_t N, int32_t n_pd, const double* transforms,
                     uint8_t* masks, void* stream) {
    if (!coeffs || !transforms || !masks || N < 2 || n_pd < 0) return MEM_ERR_INVALID;
    if (N > kMaxSmemN) return MEM_ERR_UNSUPPORTED;
    if (n_pd == 0) return MEM_OK;
    dim3 grid((unsigned)((N * N + 127) / 128), (unsigned)n_pd);
    mask_project_kernel<<<grid, 128, 0, (cudaStream_t)stream>>>(coeffs, N, transforms, masks);
    MEM_LAUNCH_CHECK();
    return MEM_OK;
}

}  // extern "C"
