// The compile-time periodic cubic B-spline rotation of an N x N image in shared memory
// (N = 64, 128), shared by the rotation kernel (prologue.cu) and the fused per-image kernel
// (image_fft.cu): the register-segment prefilter, the paired-FP32 4x4 tap sampling and one
// rotation of a whole image into per-thread runs of samples.  See prologue.cu for the
// restatement of rotatefill.op (modules/rotatefill.py:21-41) as this rotation.
#pragma once
#include "mem_internal.cuh"

namespace mem {
namespace rot {

constexpr float kZ1 = -0.26794919243112270f;     // sqrt(3) - 2, cubic B-spline pole

__device__ __forceinline__ float mask_ref(int r, int c, int N) {
    // annularMask.op(0, N/2, N, N) (annularMask.py:19-32): centre (N/2 - 1, N/2), radius N/2
    const float h = 0.5f * (float)N;
    const float x = (float)r - h + 1.0f, y = (float)c - h;
    return (x * x + y * y < h * h) ? 1.0f : 0.0f;
}

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


// Row stride of the coefficient image in the compile-time kernels: >= N + 3 (halo) and = 1 mod 32,
// so that the bank of tap (ix, iy) is (ix + iy) mod 32; a warp's 32 samples along a line whose
// direction has components of one sign then meet at most about two to a bank.
template <int N>
__host__ __device__ constexpr int rot_stride() {
    return ((N + 3 + 30) / 32) * 32 + 1;
}

template <int NT, int N>
__host__ __device__ constexpr int rot_nseg() {
    return (NT / N < N / 8) ? NT / N : N / 8;
}

template <int K>
__device__ constexpr float z1_pow() {
    float p = 1.f;
    for (int i = 0; i < K; ++i) p *= kZ1;
    return p;
}

// The periodic cubic B-spline prefilter along one axis, with each line split into NSEG segments
// of SEG >= 8 samples, one thread per segment holding it in registers.  Causal pass
// c+[k] = x[k] + z1 c+[k-1]: the thread first forms its segment's end state from zero,
// E = sum_k z1^(SEG-1-k) x[k]; the state entering segment g is sum_m z1^(SEG (m-1)) E[g-m] over
// the CT = ceil(32 / SEG) previous segments (the rest of the periodic sum is below
// z1^32 = 5e-19 of it); the recursion then runs from that state.  The anticausal pass c-[k] = c+[k] + z1 c-[k+1] does the
// same from the segment's end, and the output is -6 z1 c-[k].  Each sample is read and written
// once; segment states go through carry[] (2 NSEG N floats).  FROM_REGS: the thread's segment
// is taken from vin[] (a rotation's samples, see rotate_once) instead of shared memory.
template <int NT, int N, int AXIS, bool FROM_REGS = false>
__device__ __forceinline__ void prefilter_fixed(float* s, float* carry,
                                                const float* vin = nullptr) {
    constexpr int P = rot_stride<N>();
    constexpr int NSEG = rot_nseg<NT, N>();
    constexpr int SEG = N / NSEG, LINES = N * NSEG;
    constexpr int CT = (32 + SEG - 1) / SEG;
    static_assert(SEG >= 8 && N % NSEG == 0, "segments of at least 8 samples");
    constexpr int SK = AXIS == 0 ? 1 : P, SL = AXIS == 0 ? P : 1;
    constexpr float zseg = z1_pow<SEG>();
    constexpr float gain = -6.0f * kZ1;
    const int t = threadIdx.x;
    const bool active = LINES >= NT || t < LINES;     // a constant when every thread has a segment
    const int line = t % N, g = t / N;
    float* b0 = s + line * SL + g * SEG * SK;
    float* carry_c = carry;                 // [NSEG][N] causal end states
    float* carry_a = carry + NSEG * N;      // [NSEG][N] anticausal start states
    float v[SEG];
    if (active) {
        float e = 0.f;
#pragma unroll
        for (int k = 0; k < SEG; ++k) {
            v[k] = FROM_REGS ? vin[k] : b0[k * SK];
            e = fmaf(kZ1, e, v[k]);
        }
        carry_c[g * N + line] = e;
    }
    __syncthreads();
    if (active) {
        float c = 0.f;
#pragma unroll
        for (int m = CT; m >= 1; --m)
            c = fmaf(zseg, c, carry_c[((g + CT * NSEG - m) % NSEG) * N + line]);
#pragma unroll
        for (int k = 0; k < SEG; ++k) {
            c = fmaf(kZ1, c, v[k]);
            v[k] = c;
        }
        float e = 0.f;
#pragma unroll
        for (int k = SEG - 1; k >= 0; --k) e = fmaf(kZ1, e, v[k]);
        carry_a[g * N + line] = e;
    }
    __syncthreads();
    if (active) {
        float c = 0.f;
#pragma unroll
        for (int m = CT; m >= 1; --m) c = fmaf(zseg, c, carry_a[((g + m) % NSEG) * N + line]);
#pragma unroll
        for (int k = SEG - 1; k >= 0; --k) {
            c = fmaf(kZ1, c, v[k]);
            b0[k * SK] = gain * c;
        }
    }
    __syncthreads();
}

// Cubic B-spline weights of the 4-tap window at fractional offset t in [0, 1)
__device__ __forceinline__ void bspline_w(float t, float w[4]) {
    const float u = 1.0f - t;
    const float t2 = t * t, u2 = u * u;
    w[0] = (1.0f / 6.0f) * u2 * u;
    w[3] = (1.0f / 6.0f) * t2 * t;
    w[1] = (2.0f / 3.0f) - t2 * (1.0f - 0.5f * t);
    w[2] = (2.0f / 3.0f) - u2 * (1.0f - 0.5f * u);
}

// Two output samples a, b at once with paired FP32 instructions (fma.rn.f32x2 and friends);
// per sample the same operations in the same order as bspline_w / sample_fixed.
__device__ __forceinline__ void bspline_w2(float2 t, float2 w[4]) {
    const float2 one = make_float2(1.f, 1.f), sixth = make_float2(1.f / 6.f, 1.f / 6.f);
    const float2 two3 = make_float2(2.f / 3.f, 2.f / 3.f), half = make_float2(0.5f, 0.5f);
    const float2 mone = make_float2(-1.f, -1.f);
    const float2 u = __ffma2_rn(t, mone, one);
    const float2 t2 = __fmul2_rn(t, t), u2 = __fmul2_rn(u, u);
    w[0] = __fmul2_rn(__fmul2_rn(sixth, u2), u);
    w[3] = __fmul2_rn(__fmul2_rn(sixth, t2), t);
    // 2/3 - t^2 (1 - t/2) = 2/3 + t^2 (t/2 - 1)
    w[1] = __ffma2_rn(t2, __ffma2_rn(half, t, mone), two3);
    w[2] = __ffma2_rn(u2, __ffma2_rn(half, u, mone), two3);
}

template <int N>
__device__ __forceinline__ float2 sample_fixed2(const float* s, int64_t XA, int64_t YA, int64_t XB,
                                                int64_t YB) {
    constexpr int P = rot_stride<N>();
    const float2 k32 = make_float2(2.3283064365386963e-10f, 2.3283064365386963e-10f);
    const float2 tx = __fmul2_rn(make_float2((float)(uint32_t)(XA & 0xffffffffll),
                                             (float)(uint32_t)(XB & 0xffffffffll)), k32);
    const float2 ty = __fmul2_rn(make_float2((float)(uint32_t)(YA & 0xffffffffll),
                                             (float)(uint32_t)(YB & 0xffffffffll)), k32);
    float2 wx[4], wy[4];
    bspline_w2(tx, wx);
    bspline_w2(ty, wy);
    const float* a = s + ((int)(XA >> 32) & (N - 1)) * P + ((int)(YA >> 32) & (N - 1));
    const float* b = s + ((int)(XB >> 32) & (N - 1)) * P + ((int)(YB >> 32) & (N - 1));
    float2 acc = make_float2(0.f, 0.f);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        float2 v = __fmul2_rn(wy[0], make_float2(a[i * P], b[i * P]));
        v = __ffma2_rn(wy[1], make_float2(a[i * P + 1], b[i * P + 1]), v);
        v = __ffma2_rn(wy[2], make_float2(a[i * P + 2], b[i * P + 2]), v);
        v = __ffma2_rn(wy[3], make_float2(a[i * P + 3], b[i * P + 3]), v);
        acc = __ffma2_rn(wx[i], v, acc);
    }
    return acc;
}

// One rotation of the coefficient image in smem into keep[]: thread t has u = t % N and
// g = t / N; it samples the MAXV outputs (r, c) = (g MAXV + k, u) when the lanes run along
// output rows (lane step (sin, cos) in (x, y)), or (u, g MAXV + k) when they run along output
// columns (lane step (cos, -sin)) -- whichever step has components of one sign.  keep[] is then
// segment g of column u (rows) or of row u (columns): the segment prefilter_fixed gives thread t
// along axis 1 or 0.  Returns whether the lanes run along columns.
template <int NT, int N>
__device__ __forceinline__ bool rotate_once(const float* s, const RotConst& Q, float* keep) {
    constexpr int R = NT / N, MAXV = N / R;
    constexpr int64_t kOne = 1ll << 32;
    const int u = threadIdx.x % N, v0 = (threadIdx.x / N) * MAXV;
    const bool along_cols = (Q.rc > 0) != (Q.rs > 0);
    const int r = along_cols ? u : v0, c = along_cols ? v0 : u;
    int64_t X = Q.bx - kOne + (int64_t)r * Q.rc + (int64_t)c * Q.rs;
    int64_t Y = Q.by - kOne - (int64_t)r * Q.rs + (int64_t)c * Q.rc;
    const int64_t dX = along_cols ? Q.rs : Q.rc;
    const int64_t dY = along_cols ? Q.rc : -Q.rs;
#pragma unroll
    for (int k = 0; k < MAXV; k += 2) {
        const float2 v = sample_fixed2<N>(s, X, Y, X + dX, Y + dY);
        keep[k] = v.x;
        keep[k + 1] = v.y;
        X += 2 * dX;
        Y += 2 * dY;
    }
    return along_cols;
}


// Mask and both rotations of one image (every thread of the CTA calls it; rot[] in shared
// memory, visible to all threads after the first prefilter barrier): xi is the low-passed image
// in storage orientation (read once, thread t's first prefilter segment straight from global
// memory: image column t % N, rows (t / N) MAXV .. + MAXV - 1, lanes on consecutive columns:
// coalesced), out receives imgAll.  COHERENT: xi was written earlier in the same kernel, so it
// is read through L2 (ld.global.cg) rather than the read-only path.
template <int NT, int N, bool COHERENT>
__device__ __forceinline__ void rotate_image(const float* __restrict__ xi, float* __restrict__ out,
                                             float* s, float* carry, const RotConst* rot) {
    constexpr int P = rot_stride<N>(), NN = N * N, R = NT / N, MAXV = N / R;
    static_assert(MAXV == N / rot_nseg<NT, N>(), "a rotation's samples are one prefilter segment");
    float keep[MAXV];
    {
        const int line = threadIdx.x % N, a0 = (threadIdx.x / N) * MAXV;
#pragma unroll
        for (int k = 0; k < MAXV; ++k) {
            const float x = COHERENT ? __ldcg(xi + (a0 + k) * N + line) : xi[(a0 + k) * N + line];
            keep[k] = x * mask_ref(line, a0 + k, N);
        }
    }
    prefilter_fixed<NT, N, 0, true>(s, carry, keep);
    prefilter_fixed<NT, N, 1>(s, carry);
    fill_halo<NT>(s, N, P);
    // the second prefilter starts on the axis of the first rotation's samples, from registers
    // (the prefilter's barriers precede its stores, so every thread has finished sampling)
    if (rotate_once<NT, N>(s, rot[0], keep)) {
        prefilter_fixed<NT, N, 0, true>(s, carry, keep);
        prefilter_fixed<NT, N, 1>(s, carry);
    } else {
        prefilter_fixed<NT, N, 1, true>(s, carry, keep);
        prefilter_fixed<NT, N, 0>(s, carry);
    }
    fill_halo<NT>(s, N, P);
    const bool along_cols = rotate_once<NT, N>(s, rot[1], keep);
    const int u = threadIdx.x % N, v0 = (threadIdx.x / N) * MAXV;
    if (!along_cols) {
        // keep[k] is output (v0 + k, u): coalesced stores without staging
#pragma unroll
        for (int k = 0; k < MAXV; ++k) out[(v0 + k) * N + u] = keep[k];
        return;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < MAXV; ++k) s[u * P + v0 + k] = keep[k];     // output (u, v0 + k)
    __syncthreads();
    for (int p = threadIdx.x; p < NN; p += NT) out[p] = s[(p / N) * P + p % N];
}

}  // namespace rot
}  // namespace mem
