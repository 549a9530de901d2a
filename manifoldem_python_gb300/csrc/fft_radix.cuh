// Small in-register DFTs (lengths 4, 8, 16) for the shared-memory image transforms.
//
// dft<R, DIR>(v) replaces v[0..R) by  X[k] = sum_n v[n] exp(-DIR 2 pi i n k / R)
// (DIR = +1 forward, -1 inverse, unnormalised), natural order in and out.  Length 8 and 16 are
// radix-2 decimation in time over two half-length DFTs; the constant twiddles are cos/sin of
// multiples of pi/8, written out to float precision.  The header also compiles as host C++ so
// that the butterflies can be checked against numpy without a GPU.
#pragma once

#include <vector_functions.h>
#include <vector_types.h>

#if defined(__CUDACC__)
#define MEM_HD __host__ __device__ __forceinline__
#else
#define MEM_HD inline
#endif

namespace mem {
namespace fft {

// complex add / subtract: one paired FP32 instruction each on sm_100+ devices (the same IEEE
// operation per component; a - b as fma(b, -1, a), which is exact in the product)
MEM_HD float2 cadd(float2 a, float2 b) {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
    return __fadd2_rn(a, b);
#else
    return make_float2(a.x + b.x, a.y + b.y);
#endif
}
MEM_HD float2 csub(float2 a, float2 b) {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
    return __ffma2_rn(b, make_float2(-1.f, -1.f), a);
#else
    return make_float2(a.x - b.x, a.y - b.y);
#endif
}
MEM_HD float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
MEM_HD float2 cmulc(float2 a, float2 b) {
    return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
// a * (-DIR i)
template <int DIR>
MEM_HD float2 rot90(float2 a) {
    return DIR > 0 ? make_float2(a.y, -a.x) : make_float2(-a.y, a.x);
}
// a * exp(-DIR i pi k / 8) for a compile-time k in [0, 8)
template <int DIR, int K>
MEM_HD float2 w16(float2 a) {
    constexpr float c1 = 0.923879532511286756f;     // cos(pi/8)
    constexpr float s1 = 0.382683432365089772f;     // sin(pi/8)
    constexpr float c2 = 0.707106781186547524f;     // cos(pi/4)
    constexpr float cs[8] = {1.f, c1, c2, s1, 0.f, -s1, -c2, -c1};
    constexpr float sn[8] = {0.f, s1, c2, c1, 1.f, c1, c2, s1};
    if (K == 0) return a;
    if (K == 4) return rot90<DIR>(a);
    return cmul(a, make_float2(cs[K], -DIR * sn[K]));
}

template <int DIR>
MEM_HD void dft4(float2& a0, float2& a1, float2& a2, float2& a3) {
    const float2 t0 = cadd(a0, a2), t1 = csub(a0, a2);
    const float2 t2 = cadd(a1, a3), t3 = rot90<DIR>(csub(a1, a3));
    a0 = cadd(t0, t2);
    a2 = csub(t0, t2);
    a1 = cadd(t1, t3);
    a3 = csub(t1, t3);
}

template <int DIR>
MEM_HD void dft8(float2* v) {
    float2 e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
    float2 o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
    dft4<DIR>(e0, e1, e2, e3);
    dft4<DIR>(o0, o1, o2, o3);
    o1 = w16<DIR, 2>(o1);
    o2 = w16<DIR, 4>(o2);
    o3 = w16<DIR, 6>(o3);
    v[0] = cadd(e0, o0);
    v[4] = csub(e0, o0);
    v[1] = cadd(e1, o1);
    v[5] = csub(e1, o1);
    v[2] = cadd(e2, o2);
    v[6] = csub(e2, o2);
    v[3] = cadd(e3, o3);
    v[7] = csub(e3, o3);
}

template <int DIR>
MEM_HD void dft16(float2* v) {
    float2 e[8], o[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        e[j] = v[2 * j];
        o[j] = v[2 * j + 1];
    }
    dft8<DIR>(e);
    dft8<DIR>(o);
    o[1] = w16<DIR, 1>(o[1]);
    o[2] = w16<DIR, 2>(o[2]);
    o[3] = w16<DIR, 3>(o[3]);
    o[4] = w16<DIR, 4>(o[4]);
    o[5] = w16<DIR, 5>(o[5]);
    o[6] = w16<DIR, 6>(o[6]);
    o[7] = w16<DIR, 7>(o[7]);
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        v[k] = cadd(e[k], o[k]);
        v[k + 8] = csub(e[k], o[k]);
    }
}

template <int R, int DIR>
MEM_HD void dft(float2* v) {
    static_assert(R == 4 || R == 8 || R == 16, "dft length");
    if (R == 4) dft4<DIR>(v[0], v[1], v[2], v[3]);
    if (R == 8) dft8<DIR>(v);
    if (R == 16) dft16<DIR>(v);
}

}  // namespace fft
}  // namespace mem
