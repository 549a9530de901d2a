// Host build of the in-register DFTs (manifoldem_python_gb300/csrc/fft_radix.cuh): prints, for
// every length and direction, the input and output vectors as "R DIR re im re im ..." lines.
#include <cmath>
#include <cstdio>

#include "fft_radix.cuh"

template <int R, int DIR>
static void run(int trial) {
    float2 v[R];
    for (int n = 0; n < R; ++n)
        v[n] = make_float2(std::sin(0.37f * n + 1.1f * trial) + 0.25f * trial,
                           std::cos(0.71f * n * n + 0.3f * trial) - 0.5f);
    std::printf("in %d %d", R, DIR);
    for (int n = 0; n < R; ++n) std::printf(" %.9e %.9e", v[n].x, v[n].y);
    std::printf("\n");
    mem::fft::dft<R, DIR>(v);
    std::printf("out %d %d", R, DIR);
    for (int n = 0; n < R; ++n) std::printf(" %.9e %.9e", v[n].x, v[n].y);
    std::printf("\n");
}

int main() {
    for (int trial = 0; trial < 3; ++trial) {
        run<4, 1>(trial);
        run<4, -1>(trial);
        run<8, 1>(trial);
        run<8, -1>(trial);
        run<16, 1>(trial);
        run<16, -1>(trial);
    }
    return 0;
}
