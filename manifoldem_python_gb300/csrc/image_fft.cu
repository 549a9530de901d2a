// Shared-memory 2D real FFTs of 32x32, 64x64 and 128x128 images, one CTA per image, and the
// three kernels built from them:
//   lowpass_fft_kernel   gather + conjugate flip + background normalisation + Butterworth/Gauss
//                        low-pass (reference modules/getDistanceCTF_local_Conj9combinedS2.py
//                        :245-293), one HBM read and one HBM write per image;
//   spectrum_fft_kernel  F = fft2(imgAll) (:369), image -> half-plane spectrum [N][N/2+1];
//   inverse_fft_kernel   half-plane spectrum -> real image (imgAllFlip :375-378, the averages
//                        :383-389), unnormalised like a C2R transform.
// The half-plane layout and scaling are those of a cuFFT R2C/C2R pair, so the kernels and cuFFT
// are interchangeable stage by stage.
//
// The real 2D transform:
//   rows:     two real rows (2p, 2p+1) form one complex row Z_p = x_2p + i x_2p+1 (N/2 rows of
//             N-point complex FFTs);
//   columns:  the row spectra are separated, X_2p[k] = (Z_p[k] + conj Z_p[N-k]) / 2,
//             X_2p+1[k] = (Z_p[k] - conj Z_p[N-k]) / 2i, for k = 1..N/2-1, and the two real
//             columns k = 0 and k = N/2 are packed into one complex column X[0] + i X[N/2]:
//             N/2 columns of N-point complex FFTs.  The packed column's spectrum Y holds
//             S0 = (Y[j] + conj Y[-j]) / 2 and S_{N/2} = (Y[j] - conj Y[-j]) / 2i.
// Every N-point FFT is a four-step R1 x R2 transform done in registers: pass 1 takes elements
// t + R2 m (m < R1), a length-R1 DFT and the twiddle exp(-2 pi i t k1 / N), written back to the
// same places; pass 2 takes the R2 contiguous elements R2 k1 + t and a length-R2 DFT, written
// back in place, so a spectrum is held in digit-reversed order (frequency k1 + R1 k2 at
// position R2 k1 + k2) and the inverse passes read it in that order.  The row stage and the
// column stage share one buffer: element a of column c lives in pair-row a/2 at the position
// of frequency c (a even) or N-c (a odd; N/2 for the packed column), the same slots that hold
// the row spectra it is computed from, so every pass is in place within a thread.  Each warp
// owns 8 pair-rows and 8 columns, so only the row<->column hand-overs need a block barrier.
// The position swizzle makes every shared-memory access of the four pass shapes conflict-free
// for N = 128.
#include <algorithm>

#include "fft_radix.cuh"
#include "mem_internal.cuh"
#include "rotate_fixed.cuh"

namespace mem {
namespace {

using fft::cmul;
using fft::cmulc;

template <int N>
struct FftShape;
template <>
struct FftShape<128> {
    static constexpr int R1 = 8, R2 = 16;
};
template <>
struct FftShape<64> {
    static constexpr int R1 = 8, R2 = 8;
};
template <>
struct FftShape<32> {
    static constexpr int R1 = 4, R2 = 8;
};

__device__ __forceinline__ float bg_weight(int r, int c, int N) {
    // 1 - annularMask.op(0, N/2, N, N) (annularMask.py:19-32): centre (N/2 - 1, N/2), radius N/2
    const float h = 0.5f * (float)N;
    const float x = (float)r - h + 1.0f, y = (float)c - h;
    return (x * x + y * y < h * h) ? 0.0f : 1.0f;
}

// Kahan-compensated float accumulator
struct KSumF {
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

// The stages of the transform.  Thread mapping: warp w owns pair-rows and columns 8w..8w+7;
// the "pass 1" shape gives each lane IT1 tasks (row or column, t < R2), the "pass 2" shape IT2
// tasks (row or column, k1 < R1).
template <int N>
struct Fft2 {
    static constexpr int R1 = FftShape<N>::R1, R2 = FftShape<N>::R2, H = N / 2, NT = 2 * N;
    static constexpr int IT1 = R2 / 4, IT2 = R1 / 4, LP1 = 32 / R2, LP2 = 32 / R1;
    static constexpr int HS = H + 1;                   // half-plane row length

    // storage index of (pair-row p, position q)
    static __device__ __forceinline__ int addr(int p, int q) {
        return p * N + (q ^ (((q >> 4) * 9) & 15) ^ (((p & 7) ^ (p >> 3)) & 15));
    }
    // position of frequency k in a digit-reversed spectrum
    static __device__ __forceinline__ int pos(int k) { return R2 * (k % R1) + k / R1; }
    static __device__ __forceinline__ int warp() { return threadIdx.x >> 5; }
    static __device__ __forceinline__ int lane() { return threadIdx.x & 31; }

    // W[k] = exp(-2 pi i k / N), k < N, from the table exp(-2 pi i k / N), k <= N/2
    static __device__ __forceinline__ void twiddles(float2* W, const float2* __restrict__ twid) {
        for (int k = threadIdx.x; k < N; k += NT) {
            const float2 v = twid[k <= H ? k : k - H];
            W[k] = k <= H ? v : make_float2(-v.x, -v.y);
        }
    }

    // image rows (2p, 2p+1) -> Z_p at natural positions (pass-1 shape; no statistics);
    // COHERENT: src was written earlier in the same kernel (loads through L2, not the
    // read-only path)
    template <bool COHERENT = false>
    static __device__ __forceinline__ void load_rows(float2* S, const float* __restrict__ src) {
        const int w = warp(), l = lane();
        auto ld = [&](const float* a) { return COHERENT ? __ldcg(a) : __ldg(a); };
#pragma unroll 1
        for (int i = 0; i < IT1; ++i) {
            const int p = 8 * w + LP1 * i + l / R2, t = l % R2;
#pragma unroll
            for (int m = 0; m < R1; ++m) {
                const int b = t + R2 * m;
                S[addr(p, b)] = make_float2(ld(src + (2 * p) * N + b),
                                            ld(src + (2 * p + 1) * N + b));
            }
        }
    }

    // forward row transforms; pass 1 optionally normalises (x - mean) * inv on load
    template <bool NORM>
    static __device__ __forceinline__ void rows_forward(float2* S, const float2* W, float mean,
                                                        float inv) {
        const int w = warp(), l = lane();
#pragma unroll
        for (int i = 0; i < IT1; ++i) {
            const int p = 8 * w + LP1 * i + l / R2, t = l % R2;
            float2 v[R1];
#pragma unroll
            for (int m = 0; m < R1; ++m) {
                const float2 z = S[addr(p, t + R2 * m)];
                v[m] = NORM ? make_float2((z.x - mean) * inv, (z.y - mean) * inv) : z;
            }
            fft::dft<R1, 1>(v);
#pragma unroll
            for (int k1 = 0; k1 < R1; ++k1)
                S[addr(p, t + R2 * k1)] = k1 ? cmul(v[k1], W[t * k1]) : v[k1];
        }
        __syncwarp();
#pragma unroll
        for (int i = 0; i < IT2; ++i) {
            const int p = 8 * w + LP2 * i + l / R1, k1 = l % R1;
            float2 v[R2];
#pragma unroll
            for (int t = 0; t < R2; ++t) v[t] = S[addr(p, R2 * k1 + t)];
            fft::dft<R2, 1>(v);
#pragma unroll
            for (int k2 = 0; k2 < R2; ++k2) S[addr(p, R2 * k1 + k2)] = v[k2];
        }
    }

    // column pass 1: separate the paired rows (partner lane l^1 holds the other slot),
    // length-R1 DFT over m, twiddle
    static __device__ __forceinline__ void cols_forward1(float2* S, const float2* W) {
        const int w = warp(), l = lane();
#pragma unroll
        for (int i = 0; i < IT1; ++i) {
            const int c = 8 * w + LP1 * i + l / R2, t = l % R2;
            const bool odd = t & 1;
            const int q = pos(odd ? (c == 0 ? H : N - c) : c);
            float2 v[R1];
#pragma unroll
            for (int m = 0; m < R1; ++m) v[m] = S[addr((t + R2 * m) >> 1, q)];
#pragma unroll
            for (int m = 0; m < R1; ++m) {
                const float ux = __shfl_xor_sync(0xffffffffu, v[m].x, 1);
                const float uy = __shfl_xor_sync(0xffffffffu, v[m].y, 1);
                float2 x;
                if (c == 0)
                    x = odd ? make_float2(uy, v[m].y) : make_float2(v[m].x, ux);
                else
                    x = odd ? make_float2(0.5f * (uy + v[m].y), 0.5f * (v[m].x - ux))
                            : make_float2(0.5f * (v[m].x + ux), 0.5f * (v[m].y - uy));
                v[m] = x;
            }
            fft::dft<R1, 1>(v);
#pragma unroll
            for (int k1 = 0; k1 < R1; ++k1)
                S[addr((t + R2 * k1) >> 1, q)] = k1 ? cmul(v[k1], W[t * k1]) : v[k1];
        }
    }

    // column pass 2 of the forward transform: v[k2] = Y[k1 + R1 k2] of column c
    static __device__ __forceinline__ void cols_forward2_load(const float2* S, int c, int k1,
                                                              float2* v) {
        const int q0 = pos(c), q1 = pos(c == 0 ? H : N - c);
#pragma unroll
        for (int t = 0; t < R2; ++t) v[t] = S[addr((R2 * k1 + t) >> 1, (t & 1) ? q1 : q0)];
        fft::dft<R2, 1>(v);
    }

    // Y[-j] for j = k1 + R1 k2 of the packed column: lane k1' = (R1 - k1) mod R1 of the same
    // column holds it at k2' = R2 - 1 - k2 (k1 > 0); this lane at (R2 - k2) mod R2 (k1 = 0).
    // Every lane of the warp must call it (shuffles).
    template <int K2>
    static __device__ __forceinline__ float2 mirror(const float2* v, int k1) {
        const int srcl = (lane() / R1) * R1 + (R1 - k1) % R1;
        const float2 o = v[R2 - 1 - K2];
        const float px = __shfl_sync(0xffffffffu, o.x, srcl);
        const float py = __shfl_sync(0xffffffffu, o.y, srcl);
        return k1 == 0 ? v[(R2 - K2) % R2] : make_float2(px, py);
    }

    // inverse pass 1 of column c from the spectrum in registers: length-R2 inverse DFT and
    // conjugate twiddle, stored in place
    static __device__ __forceinline__ void cols_inverse1_store(float2* S, const float2* W, int c,
                                                               int k1, float2* v) {
        const int q0 = pos(c), q1 = pos(c == 0 ? H : N - c);
        fft::dft<R2, -1>(v);
#pragma unroll
        for (int t = 0; t < R2; ++t)
            S[addr((R2 * k1 + t) >> 1, (t & 1) ? q1 : q0)] = k1 ? cmulc(v[t], W[t * k1]) : v[t];
    }

    // column pass 2 with the low-pass: forward DFT, multiply by G/N^2 (gtab [N][N/2+1];
    // G(j, .) = G(N-j, .)), inverse DFT
    static __device__ __forceinline__ void cols_filter(float2* S, const float2* W,
                                                       const float* __restrict__ gtab) {
        const int w = warp(), l = lane();
#pragma unroll
        for (int i = 0; i < IT2; ++i) {
            const int c = 8 * w + LP2 * i + l / R1, k1 = l % R1;
            float2 v[R2];
            cols_forward2_load(S, c, k1, v);
            if (w == 0 && i == 0) {
                // packed column (c = 0): Y'[j] = Y[j] (G0 + Gh)/2 + conj Y[-j] (G0 - Gh)/2.
                // Its lanes leave their spectrum values in the column's own slots (read above,
                // rewritten by cols_inverse1_store below; only this warp touches them) and read
                // the mirrors Y[-j] back from there, so the filter is applied in place in v[]
                // with no second register array.
                const int q0 = pos(0), q1 = pos(H);
                auto slot = [&](int kk1, int k2) {
                    return addr((R2 * kk1 + k2) >> 1, (k2 & 1) ? q1 : q0);
                };
                if (c == 0) {
#pragma unroll
                    for (int k2 = 0; k2 < R2; ++k2) S[slot(k1, k2)] = v[k2];
                }
                __syncwarp();
                if (c == 0) {
                    // Y[-j] for j = k1 + R1 k2: lane (R1 - k1) mod R1's value at R2 - 1 - k2
                    // (k1 > 0), this lane's at (R2 - k2) mod R2 (k1 = 0)
                    const int mk1 = (R1 - k1) % R1;
#pragma unroll
                    for (int k2 = 0; k2 < R2; ++k2) {
                        const float2 m =
                            S[slot(mk1, k1 == 0 ? (R2 - k2) % R2 : R2 - 1 - k2)];
                        const int j = k1 + R1 * k2;
                        const int fa = min(j, N - j);
                        const float g0 = __ldg(gtab + fa * HS), gh = __ldg(gtab + fa * HS + H);
                        const float gp = 0.5f * (g0 + gh), gm = 0.5f * (g0 - gh);
                        v[k2] = make_float2(v[k2].x * gp + m.x * gm, v[k2].y * gp - m.y * gm);
                    }
                } else {
#pragma unroll
                    for (int k2 = 0; k2 < R2; ++k2) {
                        const int j = k1 + R1 * k2;
                        const float g = __ldg(gtab + min(j, N - j) * HS + c);
                        v[k2] = make_float2(v[k2].x * g, v[k2].y * g);
                    }
                }
                __syncwarp();           // every mirror read before the slots are rewritten
            } else {
#pragma unroll
                for (int k2 = 0; k2 < R2; ++k2) {
                    const int j = k1 + R1 * k2;
                    const float g = __ldg(gtab + min(j, N - j) * HS + c);
                    v[k2] = make_float2(v[k2].x * g, v[k2].y * g);
                }
            }
            cols_inverse1_store(S, W, c, k1, v);
        }
    }

    // Row-by-row access to the digit-reversed column spectra: thread t owns column c = t % H
    // and rows j = j0 + 4 i (j0 = t / H < 4, i < N/4).  For those rows the digit-reversed
    // position is R2 j0 + delta(i) with a compile-time delta, so the slot's pair-row, parity and
    // most of its swizzle are constants of the unrolled loop.
    static constexpr int kRowsPerThread = N / 4;
    static_assert(NT == 4 * H && R1 % 4 == 0, "row walk: four row phases, R1 a multiple of 4");
    static __device__ __forceinline__ int rdelta(int i) {
        return 4 * R2 * (i % (R1 / 4)) + i / (R1 / 4);
    }
    // storage index of (column c, row j0 + 4 i); q0 = pos(c), q1 = pos of c's odd slot
    static __device__ __forceinline__ int row_slot(int j0, int i, int q0, int q1) {
        const int a = R2 * j0 + rdelta(i);
        return addr(a >> 1, (rdelta(i) & 1) ? q1 : q0);
    }

    // the packed column's half-plane values from its spectrum Y (lanes of one column)
    template <int K2>
    static __device__ __forceinline__ void unpack_packed(const float2* v, int k1, int c,
                                                         float2* __restrict__ spec) {
        if constexpr (K2 < R2) {
            const float2 m = mirror<K2>(v, k1);
            if (c == 0) {
                const int j = k1 + R1 * K2;
                spec[j * HS] = make_float2(0.5f * (v[K2].x + m.x), 0.5f * (v[K2].y - m.y));
                spec[j * HS + H] = make_float2(0.5f * (v[K2].y + m.y), 0.5f * (m.x - v[K2].x));
            }
            unpack_packed<K2 + 1>(v, k1, c, spec);
        }
    }

    // column pass 2 of the forward transform, written out as the half-plane spectrum straight
    // from registers (row segments of 32 bytes, merged in L2; measured faster than staging the
    // rows through shared memory for coalesced stores)
    static __device__ __forceinline__ void cols_spectrum_out(const float2* S,
                                                             float2* __restrict__ spec) {
        const int w = warp(), l = lane();
#pragma unroll
        for (int i = 0; i < IT2; ++i) {
            const int c = 8 * w + LP2 * i + l / R1, k1 = l % R1;
            float2 v[R2];
            cols_forward2_load(S, c, k1, v);
            if (w == 0 && i == 0) {
                unpack_packed<0>(v, k1, c, spec);
                if (c == 0) continue;
            }
#pragma unroll
            for (int k2 = 0; k2 < R2; ++k2) spec[(k1 + R1 * k2) * HS + c] = v[k2];
        }
    }

    // inverse column pass 1 from a half-plane spectrum in global memory, read row by row
    // (coalesced) into the columns' digit-reversed slots; SIGNED multiplies element (j, c) by
    // sign(C(m)) / N^2, m = min(j, N-j)^2 + c^2 (the phase flip)
    template <bool SIGNED>
    static __device__ __forceinline__ float2 spec_at(const float2* __restrict__ spec, int j, int c,
                                                     uint64_t qf, const CtfConst& cc) {
        const float2 v = spec[j * HS + c];
        if (!SIGNED) return v;
        const int fa = min(j, N - j);
        const float g = (float)ctf_sign(fa * fa + c * c, qf, cc) * (1.0f / ((float)N * (float)N));
        return make_float2(g * v.x, g * v.y);
    }

    template <bool SIGNED>
    static __device__ __forceinline__ void cols_spectrum_in(float2* S, const float2* W,
                                                            const float2* __restrict__ spec,
                                                            uint64_t qf, const CtfConst& cc) {
        {
            const int c = threadIdx.x % H, j0 = threadIdx.x / H;
            const int q0 = pos(c), q1 = pos(c == 0 ? H : N - c);
#pragma unroll 8
            for (int i = 0; i < kRowsPerThread; ++i) {
                const int j = j0 + 4 * i;
                float2 y = spec_at<SIGNED>(spec, j, c, qf, cc);
                if (c == 0) {                              // S0 + i S_{N/2}
                    const float2 b = spec_at<SIGNED>(spec, j, H, qf, cc);
                    y = make_float2(y.x - b.y, y.y + b.x);
                }
                S[row_slot(j0, i, q0, q1)] = y;
            }
        }
        __syncthreads();
        const int w = warp(), l = lane();
#pragma unroll
        for (int i = 0; i < IT2; ++i) {
            const int c = 8 * w + LP2 * i + l / R1, k1 = l % R1;
            const int q0 = pos(c), q1 = pos(c == 0 ? H : N - c);
            float2 v[R2];
#pragma unroll
            for (int k2 = 0; k2 < R2; ++k2)
                v[k2] = S[addr((R2 * k1 + k2) >> 1, (k2 & 1) ? q1 : q0)];
            cols_inverse1_store(S, W, c, k1, v);
        }
    }

    // inverse column pass 2: length-R1 inverse DFT, then rebuild the paired rows
    static __device__ __forceinline__ void cols_inverse2(float2* S) {
        const int w = warp(), l = lane();
#pragma unroll
        for (int i = 0; i < IT1; ++i) {
            const int c = 8 * w + LP1 * i + l / R2, t = l % R2;
            const bool odd = t & 1;
            const int q = pos(odd ? (c == 0 ? H : N - c) : c);
            float2 v[R1];
#pragma unroll
            for (int m = 0; m < R1; ++m) v[m] = S[addr((t + R2 * m) >> 1, q)];
            fft::dft<R1, -1>(v);
#pragma unroll
            for (int m = 0; m < R1; ++m) {
                const float ux = __shfl_xor_sync(0xffffffffu, v[m].x, 1);
                const float uy = __shfl_xor_sync(0xffffffffu, v[m].y, 1);
                float2 z;
                if (c == 0)
                    z = odd ? make_float2(uy, v[m].y) : make_float2(v[m].x, ux);
                else
                    z = odd ? make_float2(ux + v[m].y, v[m].x - uy)
                            : make_float2(v[m].x - uy, v[m].y + ux);
                S[addr((t + R2 * m) >> 1, q)] = z;
            }
        }
    }

    // inverse row transforms of the digit-reversed row spectra; real part -> row 2p,
    // imaginary part -> row 2p+1 of dst
    static __device__ __forceinline__ void rows_inverse(float2* S, const float2* W,
                                                        float* __restrict__ dst) {
        const int w = warp(), l = lane();
#pragma unroll
        for (int i = 0; i < IT2; ++i) {
            const int p = 8 * w + LP2 * i + l / R1, k1 = l % R1;
            float2 v[R2];
#pragma unroll
            for (int k2 = 0; k2 < R2; ++k2) v[k2] = S[addr(p, R2 * k1 + k2)];
            fft::dft<R2, -1>(v);
#pragma unroll
            for (int t = 0; t < R2; ++t)
                S[addr(p, R2 * k1 + t)] = k1 ? cmulc(v[t], W[t * k1]) : v[t];
        }
        __syncwarp();
#pragma unroll
        for (int i = 0; i < IT1; ++i) {
            const int p = 8 * w + LP1 * i + l / R2, t = l % R2;
            float2 v[R1];
#pragma unroll
            for (int k1 = 0; k1 < R1; ++k1) v[k1] = S[addr(p, R2 * k1 + t)];
            fft::dft<R1, -1>(v);
#pragma unroll
            for (int m = 0; m < R1; ++m) {
                dst[(2 * p) * N + t + R2 * m] = v[m].x;
                dst[(2 * p + 1) * N + t + R2 * m] = v[m].y;
            }
        }
    }
};

// gather + flip + normalisation + low-pass of one image (every thread of the CTA calls it)
template <int N>
__device__ __forceinline__ void lowpass_image(
        int64_t img, float2* S, const float2* W, double* red, const float* __restrict__ stack,
        int64_t num_stack, const int64_t* __restrict__ sidx, const uint8_t* __restrict__ flip,
        const float* __restrict__ gtab, float* __restrict__ xbuf, uint32_t* __restrict__ status) {
    using F = Fft2<N>;
    constexpr int NT = F::NT, NN = N * N, R1 = F::R1, R2 = F::R2;
    const int w = F::warp(), l = F::lane();
    const int64_t s = sidx[img];
    float* dst = xbuf + img * (int64_t)NN;
    if (s < 0 || s >= num_stack) {
        if (threadIdx.x == 0) atomicOr(status, 2u);
        for (int e = threadIdx.x; e < NN; e += NT) dst[e] = __int_as_float(0x7fc00000);
        return;
    }
    const bool f = flip[img] != 0;
    const float* src = stack + s * (int64_t)NN;
    // rows (2p, 2p+1) -> Z_p at natural positions; background statistics (:277-281)
    KSumF sum, sq;
#pragma unroll 2
    for (int i = 0; i < F::IT1; ++i) {
        const int p = 8 * w + F::LP1 * i + l / R2, t = l % R2;
#pragma unroll
        for (int m = 0; m < R1; ++m) {
            const int b = t + R2 * m;
            const int bs = f ? N - 1 - b : b;
            const float x0 = __ldg(src + (2 * p) * N + bs);
            const float x1 = __ldg(src + (2 * p + 1) * N + bs);
            const float g0 = x0 * bg_weight(b, 2 * p, N), g1 = x1 * bg_weight(b, 2 * p + 1, N);
            sum.add(g0);
            sq.add(g0 * g0);
            sum.add(g1);
            sq.add(g1 * g1);
            S[F::addr(p, b)] = make_float2(x0, x1);
        }
    }
    float mean, inv;
    block_stats<NT>((double)sum.value(), (double)sq.value(), red, NN, &mean, &inv);
    F::template rows_forward<true>(S, W, mean, inv);
    __syncthreads();
    F::cols_forward1(S, W);
    __syncwarp();
    F::cols_filter(S, W, gtab);
    __syncwarp();
    F::cols_inverse2(S);
    __syncthreads();
    F::rows_inverse(S, W, dst);
}

// one image per CTA (N = 128: two CTAs per SM; a register budget for three spills 52 bytes and
// measured slower, 28.4 against 23.3 ms on config4)
template <int N>
__global__ void __launch_bounds__(2 * N, N == 128 ? 2 : 4) lowpass_fft_kernel(
        const float* __restrict__ stack, int64_t num_stack, const int64_t* __restrict__ sidx,
        const uint8_t* __restrict__ flip, const float* __restrict__ gtab,
        const float2* __restrict__ twid, float* __restrict__ xbuf, uint32_t* __restrict__ status) {
    using F = Fft2<N>;
    extern __shared__ float2 S[];                      // [N/2][N], swizzled
    __shared__ float2 W[N];
    __shared__ double red[2 * (F::NT / 32)];
    F::twiddles(W, twid);
    lowpass_image<N>(blockIdx.x, S, W, red, stack, num_stack, sidx, flip, gtab, xbuf, status);
}

template <int N>
__global__ void __launch_bounds__(2 * N, N == 128 ? 3 : 4) spectrum_fft_kernel(
        const float* __restrict__ images, const float2* __restrict__ twid,
        float2* __restrict__ spec) {
    using F = Fft2<N>;
    extern __shared__ float2 S[];
    __shared__ float2 W[N];
    const int64_t img = blockIdx.x;
    F::twiddles(W, twid);
    F::load_rows(S, images + img * (int64_t)N * N);
    __syncthreads();
    F::template rows_forward<false>(S, W, 0.f, 1.f);
    __syncthreads();
    F::cols_forward1(S, W);
    __syncwarp();
    F::cols_spectrum_out(S, spec + img * (int64_t)N * F::HS);
}

// The image stage of one image in one CTA (N = 64, 128; no volume mask): gather + conjugate
// flip + background normalisation + low-pass (lowpass_image), mask + the two periodic cubic
// B-spline rotations (rot::rotate_image), and F = fft2(imgAll) written as the half-plane
// spectrum -- the three kernels of the unfused path in one, so that the CTAs on an SM overlap
// the FFTs' latency-bound passes with the rotation's shared-memory-bound sampling.  The
// low-passed image and imgAll go through global memory (xbuf / img_out: L2-resident, read back
// by the same CTA through L2); the shared buffer is reused by each phase.
template <int N>
__global__ void __launch_bounds__(2 * N, N == 128 ? 2 : 4) image_stage_kernel(
        const float* __restrict__ stack, int64_t num_stack, const int64_t* __restrict__ sidx,
        const uint8_t* __restrict__ flip, const float* __restrict__ gtab,
        const float2* __restrict__ twid, float* xbuf, float* img_out,
        const rot::RotConst* __restrict__ rotc, float2* __restrict__ spec,
        uint32_t* __restrict__ status) {
    using F = Fft2<N>;
    constexpr int NT = 2 * N, NN = N * N;
    extern __shared__ float2 S[];                      // FFT buffer, then rotation image
    __shared__ float2 W[N];
    __shared__ double red[2 * (NT / 32)];
    __shared__ rot::RotConst rc[2];
    __shared__ float carry[2 * rot::rot_nseg<NT, N>() * N];
    const int64_t img = blockIdx.x;
    F::twiddles(W, twid);
    if (threadIdx.x < 2) rc[threadIdx.x] = rotc[2 * img + threadIdx.x];
    float* xi = xbuf + img * (int64_t)NN;
    float* out = img_out + img * (int64_t)NN;
    lowpass_image<N>(img, S, W, red, stack, num_stack, sidx, flip, gtab, xbuf, status);
    __syncthreads();                                   // xi written, S free
    rot::rotate_image<NT, N, true>(xi, out, reinterpret_cast<float*>(S), carry, rc);
    __syncthreads();                                   // imgAll written, S free
    F::template load_rows<true>(S, out);
    __syncthreads();
    F::template rows_forward<false>(S, W, 0.f, 1.f);
    __syncthreads();
    F::cols_forward1(S, W);
    __syncwarp();
    F::cols_spectrum_out(S, spec + img * (int64_t)N * F::HS);
}

template <int N, bool SIGNED>
__global__ void __launch_bounds__(2 * N, N == 128 ? 3 : 4) inverse_fft_kernel(
        const float2* __restrict__ spec, const float2* __restrict__ twid,
        float* __restrict__ images, const uint64_t* __restrict__ qfix, CtfConst cc) {
    using F = Fft2<N>;
    extern __shared__ float2 S[];
    __shared__ float2 W[N];
    const int64_t img = blockIdx.x;
    F::twiddles(W, twid);
    __syncthreads();
    F::template cols_spectrum_in<SIGNED>(S, W, spec + img * (int64_t)N * F::HS,
                                         SIGNED ? qfix[img] : 0ull, cc);
    __syncwarp();
    F::cols_inverse2(S);
    __syncthreads();
    F::rows_inverse(S, W, images + img * (int64_t)N * N);
}

template <typename K>
int prepare(K kernel, size_t smem) {
    MEM_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
    return MEM_OK;
}

}  // namespace

namespace kern {
bool smem_fft_supported(const mem_plan& P) { return P.N == 32 || P.N == 64 || P.N == 128; }

#define MEM_FFT_DISPATCH(CALL)            \
    switch (P.N) {                        \
        case 32: CALL(32); break;         \
        case 64: CALL(64); break;         \
        case 128: CALL(128); break;       \
        default: return MEM_ERR_UNSUPPORTED; \
    }

int lowpass_fused(const mem_plan& P, const mem_inputs& in, const float* gtab,
                  const float2* twid, float* xbuf, uint32_t* status, cudaStream_t s) {
    if (P.n_images == 0) return MEM_OK;
    const size_t smem = (size_t)(P.N / 2) * P.N * sizeof(float2);
#define MEM_CALL(NV)                                                                           \
    do {                                                                                       \
        if (prepare(lowpass_fft_kernel<NV>, smem) != MEM_OK) return MEM_ERR_CUDA;              \
        lowpass_fft_kernel<NV><<<(unsigned)P.n_images, 2 * NV, smem, s>>>(                     \
                in.stack, in.num_stack, in.stack_index, in.flip, gtab, twid, xbuf, status);    \
    } while (0)
    MEM_FFT_DISPATCH(MEM_CALL)
#undef MEM_CALL
    MEM_LAUNCH_CHECK();
    return MEM_OK;
}

bool image_stage_supported(const mem_plan& P) { return P.N == 64 || P.N == 128; }

int image_stage(const mem_plan& P, const mem_inputs& in, const float* gtab, const float2* twid,
                float* xbuf, float* img_out, const void* rotc, float2* spec, uint32_t* status,
                cudaStream_t s) {
    if (P.n_images == 0) return MEM_OK;
    const rot::RotConst* rc = static_cast<const rot::RotConst*>(rotc);
#define MEM_CALL(NV)                                                                           \
    do {                                                                                       \
        const size_t smem = std::max((size_t)(NV / 2) * NV * sizeof(float2),                   \
                                     (size_t)(NV + 3) * rot::rot_stride<NV>() * sizeof(float)); \
        if (prepare(image_stage_kernel<NV>, smem) != MEM_OK) return MEM_ERR_CUDA;              \
        image_stage_kernel<NV><<<(unsigned)P.n_images, 2 * NV, smem, s>>>(                     \
                in.stack, in.num_stack, in.stack_index, in.flip, gtab, twid, xbuf, img_out,    \
                rc, spec, status);                                                             \
    } while (0)
    switch (P.N) {
        case 64: MEM_CALL(64); break;
        case 128: MEM_CALL(128); break;
        default: return MEM_ERR_UNSUPPORTED;
    }
#undef MEM_CALL
    MEM_LAUNCH_CHECK();
    return MEM_OK;
}

int spectrum_fft(const mem_plan& P, int64_t count, const float* images, const float2* twid,
                 float2* spec, cudaStream_t s) {
    if (count == 0) return MEM_OK;
    const size_t smem = (size_t)(P.N / 2) * P.N * sizeof(float2);
#define MEM_CALL(NV)                                                                           \
    do {                                                                                       \
        if (prepare(spectrum_fft_kernel<NV>, smem) != MEM_OK) return MEM_ERR_CUDA;             \
        spectrum_fft_kernel<NV><<<(unsigned)count, 2 * NV, smem, s>>>(images, twid, spec);     \
    } while (0)
    MEM_FFT_DISPATCH(MEM_CALL)
#undef MEM_CALL
    MEM_LAUNCH_CHECK();
    return MEM_OK;
}

int inverse_fft(const mem_plan& P, int64_t count, const float2* spec, const float2* twid,
                float* images, const uint64_t* qf, bool signed_flip, cudaStream_t s) {
    if (count == 0) return MEM_OK;
    const size_t smem = (size_t)(P.N / 2) * P.N * sizeof(float2);
#define MEM_CALL(NV)                                                                           \
    do {                                                                                       \
        if (signed_flip) {                                                                     \
            if (prepare(inverse_fft_kernel<NV, true>, smem) != MEM_OK) return MEM_ERR_CUDA;    \
            inverse_fft_kernel<NV, true><<<(unsigned)count, 2 * NV, smem, s>>>(                \
                    spec, twid, images, qf, P.ctf);                                            \
        } else {                                                                               \
            if (prepare(inverse_fft_kernel<NV, false>, smem) != MEM_OK) return MEM_ERR_CUDA;   \
            inverse_fft_kernel<NV, false><<<(unsigned)count, 2 * NV, smem, s>>>(               \
                    spec, twid, images, qf, P.ctf);                                            \
        }                                                                                      \
    } while (0)
    MEM_FFT_DISPATCH(MEM_CALL)
#undef MEM_CALL
    MEM_LAUNCH_CHECK();
    return MEM_OK;
}
#undef MEM_FFT_DISPATCH
}  // namespace kern
}  // namespace mem
