// Internal declarations shared by the distance-stage translation units.
#pragma once

#include <cuda_runtime.h>
#include <cufft.h>
#include <cstdint>
#include <utility>
#include <vector>

#include "../../include/manifoldem_gb300.h"

namespace mem {

constexpr int kMaxSmemN = 236;      // the rotation keeps one (N+3) x (N+3)|1 float image in smem
constexpr int kMaxN = 512;          // larger boxes rotate with coefficients in global memory
constexpr int kRowBlock = 128;      // PD rows are padded to this in the feature matrix
constexpr int kKPad = 64;           // each feature block is padded to a multiple of this
constexpr int kSumChunk = 256;      // images per partial-sum item of the per-PD reductions
constexpr int kFftChunk = 8192;     // images per batched cuFFT execution

// device status word bits (first 4 bytes of the workspace)
constexpr uint32_t kStatusTimeout = 1u;
constexpr uint32_t kStatusBadIndex = 2u;
constexpr long long kDefaultWaitCycles = 4000000000ll;   // ~2 s at 2 GHz

// wait limit and withheld chunk from MEM_WAIT_CYCLES / MEM_TEST_WITHHOLD_CHUNK (tests of the
// timeout path); defaults otherwise
void wait_settings_from_env(long long* cycles, int* withhold);

// ---- per-PD table uploaded to the workspace --------------------------------------------
struct PdDev {
    int64_t img_off;     // first image of the PD
    int64_t row_off;     // first feature-matrix row of the PD (multiple of kRowBlock)
    int64_t d_off;       // first element of the PD's D block
    int32_t n;           // images in the PD
    int32_t pad;
    double  rot2_cos, rot2_sin;   // rotation by -psi_p
};

// partial-sum item: images [img_begin, img_end) of PD pd
struct SumItem {
    int32_t pd;
    int32_t pad;
    int64_t img_begin, img_end;
};

// D contraction tile: PD pd, 128-row block I, column block J of the tile's width (128 for the
// FP32 form; 128 or 256 for the split-BF16 form's classes)
struct Tile {
    int32_t pd, I, J, pad;
};

// CTF constants (phase in 64-bit fixed-point cycles; see prologue.cu)
struct CtfConst {
    uint64_t p_fix;        // frac(Cs term per m^2) * 2^64
    uint64_t d_fix;        // frac(atan(A) / 2pi) * 2^64
    double   q_scale;      // defocus cycles per m per Angstrom: lambda / (2 (N pix)^2)
    float    amp;          // sqrt(1 + A^2)
    float    env_c;        // envelope exponent per m: 1 / ((N pix)^2 2 sigma^2), 0 if none
};

// sign of the CTF at squared radius m (frequency units) for an image with defocus phase qf: the
// sign of the 64-bit fixed-point phase P m^2 - Q m - atan(A)/2pi, whose sine (times a positive
// amplitude) is the CTF
__device__ __forceinline__ int ctf_sign(int m, uint64_t qf, const CtfConst& cc) {
    const uint64_t mm = (uint32_t)m;                  // m >= 0: zero-extended
    const int64_t sph = (int64_t)(cc.p_fix * (mm * mm) - qf * mm - cc.d_fix);
    return (sph > 0) - (sph < 0);
}

// device tables of the feature layout (feature_layout): colmap [Kc_pad] = column of frequency
// slot k within the r' / s' blocks; ring features: ring R = frequencies of |k|^2 = ring_m[R],
// stored at positions ring_start[R] .. ring_start[R+1] of the ring order, pos_of[k] = position of
// frequency k, ring_of[k] = its ring; chunks [n_chunks] = (A column, B column, negate B, add the
// lo.lo product) of each 64-wide K chunk of the contraction
struct FeatTables {
    const int32_t* colmap;
    const int32_t* ring_start;
    const int32_t* ring_m;
    const int32_t* pos_of;
    const int32_t* ring_of;
    const int4* chunks;
};

struct Layout {
    size_t status, pd_table, sum_items, img_pd, img_row, tiles, tc_tiles;
    size_t item_off, qfix, rotc, gtab, pd_max, colmap, twid, ident;
    size_t xbuf, spec, feat_a, feat_b, pair_norm, partial, means, avg_spec, avg_real, cufft_work;
    size_t total;
};

}  // namespace mem

struct mem_plan {
    mem_params params;
    int32_t n_pd = 0;
    int64_t n_images = 0;
    int N = 0, Nh = 0;              // Nh = N/2 + 1
    int64_t Kc = 0, Kc_pad = 0;     // half-plane frequencies, padded to kKPad
    // feature row: [U' (Kr_pad) | V' (Kr_pad) | r' (Kc_pad) | s' (Kc_pad)], Kf columns; with ring
    // features U', V' are indexed by rings of equal |k|^2 (Kr rings), else by frequency (Kr = Kc)
    bool ring_features = true;
    int64_t Kr = 0, Kr_pad = 0, Kf = 0;
    int n_chunks = 0;
    std::vector<int32_t> ftab;      // host image of the FeatTables (int32 words)
    size_t ft_ring_start = 0, ft_ring_m = 0, ft_pos_of = 0, ft_ring_of = 0, ft_chunks = 0;
    int64_t n_rows = 0;             // feature-matrix rows (padded per PD)
    int64_t d_elems = 0, n_pairs = 0;
    std::vector<int32_t> count;
    std::vector<mem::PdDev> pd;
    std::vector<mem::SumItem> items;
    std::vector<int32_t> img_pd, img_row;
    std::vector<mem::Tile> tiles;
    std::vector<int32_t> colmap;    // feature column of frequency slot k (chunks radius-descending)
    mem::CtfConst ctf{};
    mem::Layout lay{};
    size_t cufft_work_bytes = 0;
    int device = -1;
    int num_sms = 0;
    // contraction schedule per size class (mem_plan_set_contraction) and each class's range of
    // the tile list (tiles sorted by class): (first tile, tile count)
    std::vector<mem_contraction_config> tc_classes;
    std::vector<std::pair<int, int>> tc_ranges;
    std::vector<mem::Tile> tc_tiles;   // the split-BF16 contraction's tiles (J in tile_n units)
    bool uploaded = false;
    int tc_group_chunks = 1;        // 64-wide K chunks per TMEM accumulation group (0 = all)
    bool tc_kahan = false;          // compensated register sums across groups
    bool tc_lolo = false;           // add the lo.lo product (4-term split)
    bool smem_fft = true;           // shared-memory FFT kernels instead of cuFFT (N = 32, 64, 128)
    // N = 64, 128 without a volume mask: low-pass, rotations and spectrum in one kernel
    // (MEM_FUSED_IMAGE=1; off by default: measured slower than the three kernels, see
    // image_stage_kernel)
    bool fused_image = false;
    // boxes rotated by rotate_band: 1 = N > 236 (no whole-image shared-memory kernel), 2 = also
    // N <= 236 without a compile-time kernel, 0 = never (MEM_ROT_BAND)
    int rot_band = 1;
    int rot_band_variant = 2;       // rotate_band's sampling / occupancy form (MEM_ROT_BAND_VARIANT)
    // host-to-device image copy of a split execute: the fewer SMs it occupies the less it slows
    // the concurrent computation; 8 x 1024 threads, two images per step, keep ~1 MB of loads in
    // flight, enough for the host link
    int host_load_ctas = 8;
    int host_load_threads = 1024;   // 256, 512 or 1024
                                    // with the stack in host memory
    // bounded device-side waits (the tcgen05 contraction's mbarrier waits) give up after this
    // many SM clock cycles (~2 s at 2 GHz) and set the status word's timeout bit
    long long wait_cycles = mem::kDefaultWaitCycles;
    // test of the timeout path only: the contraction's producer never loads this chunk (-1: none),
    // so the wait for it can only end by the limit above
    int test_withhold_chunk = -1;
    bool timing = false;
    bool timed_run = false;
    cudaEvent_t ev[MEM_NUM_PHASES + 1] = {};
    bool phase_ran[MEM_NUM_PHASES] = {};
    cudaEvent_t load_done = nullptr; // end of the stack-reading phase (mem_plan_execute_split)
    ~mem_plan() {
        for (auto& e : ev)
            if (e) cudaEventDestroy(e);
        if (load_done) cudaEventDestroy(load_done);
    }
};

namespace mem {

// ---- batched 2D cuFFT transforms of N x N images (abi.cu): R2C image -> half-plane [N][N/2+1]
// or C2R back, `count` transforms in chunks of kFftChunk from a per-(device, N, kind, batch) plan
// cache; work is a caller-owned area of fft_work_bytes(N, type, count) bytes
size_t fft_work_bytes(int N, cufftType type, int64_t count);
int fft_exec(int device, int N, cufftType type, int64_t count, int64_t in_stride,
             int64_t out_stride, void* in, void* out, void* work, cudaStream_t s);

// ---- host launchers of the image-side kernels (prologue.cu) ------------------------------
namespace kern {
int gather_normalize(const mem_plan& P, const mem_inputs& in, float* xbuf, uint32_t* status,
                     int64_t max_ctas, cudaStream_t s);
// raw copies of the entries' stack images into out [n_images][N][N] (ctas CTAs loop over them)
int gather_copy(const mem_plan& P, const mem_inputs& in, float* out, uint32_t* status,
                int64_t ctas, cudaStream_t s);
// multiply the half-plane spectra by the table G/N^2 written by lowpass_table
int lowpass(const mem_plan& P, float2* spec, float* gtab, cudaStream_t s);
bool smem_fft_supported(const mem_plan& P);
int lowpass_table(const mem_plan& P, float* gtab, cudaStream_t s);
int lowpass_fused(const mem_plan& P, const mem_inputs& in, const float* gtab,
                  const float2* twid, float* xbuf, uint32_t* status, cudaStream_t s);
// dst[img] = src[img] times the mask of the image's PD (in place when dst == src)
int apply_pd_mask(const mem_plan& P, const float* src, float* dst, const uint8_t* masks,
                  const int32_t* img_pd, cudaStream_t s);
// RELION read: shifted images, laid out as SPIDER stack images, into out [n_images][N][N]
int relion_shift(const mem_plan& P, const mem_inputs& in, float* out, uint32_t* status,
                 cudaStream_t s);
// shared-memory real 2D FFTs (N = 32, 64, 128) with the layout and scaling of a cuFFT R2C/C2R
int spectrum_fft(const mem_plan& P, int64_t count, const float* images, const float2* twid,
                 float2* spec, cudaStream_t s);
// signed = the phase-flip inverse: element k of image i multiplied by sign(C_i(k)) / N^2 on load
int inverse_fft(const mem_plan& P, int64_t count, const float2* spec, const float2* twid,
                float* images, const uint64_t* qf, bool signed_flip, cudaStream_t s);
// the two rotations' fixed-point constants of every image into rot_scratch (64 bytes each)
int rot_consts(const mem_plan& P, const mem_inputs& in, const PdDev* pd_table,
               const int32_t* img_pd, void* rot_scratch, cudaStream_t s);
// N = 64, 128: gather + flip + normalisation + low-pass, mask + both rotations and the spectrum
// of imgAll in one kernel (rot_consts first); img_out receives imgAll, spec the spectra
bool image_stage_supported(const mem_plan& P);
int image_stage(const mem_plan& P, const mem_inputs& in, const float* gtab, const float2* twid,
                float* xbuf, float* img_out, const void* rotc, float2* spec, uint32_t* status,
                cudaStream_t s);
// rot_scratch: 64 bytes per image (the two rotations' fixed-point constants)
int rotate(const mem_plan& P, const mem_inputs& in, float* xbuf, float* img_out,
           const PdDev* pd_table, const int32_t* img_pd, float2* spec, void* rot_scratch,
           cudaStream_t s);
// the two rotations with the coefficient image in bands of rows (64 <= N <= 512; rotate calls it
// for boxes without a shared-memory kernel); spec is the coefficient scratch
bool rotate_band_supported(int N);
int rotate_band(const mem_plan& P, float* xbuf, float2* spec, float* img_out, const void* rotc,
                cudaStream_t s);
int qfix(const mem_plan& P, const mem_inputs& in, uint64_t* qf, cudaStream_t s);
// which: 1 = S0..S2, 2 = S3..S5, 3 = all six per-PD sums
int pd_sums(const mem_plan& P, const float2* spec, const uint64_t* qf, const SumItem* items,
            float* partial, int which, cudaStream_t s);
// mode bit 1: Wiener average spectrum; bit 2: centring vectors, scale, phase-flip average
int pd_finalize(const mem_plan& P, const float* partial, const SumItem* items,
                const int32_t* item_off, const PdDev* pds, const int32_t* ring_of, float* means,
                float2* avg_spec, uint32_t* pd_max, int mode, cudaStream_t s);
int features(const mem_plan& P, float2* spec, const uint64_t* qf, const PdDev* pds,
             const int32_t* img_pd, const int32_t* img_row, const FeatTables& ft,
             const float* means, const uint32_t* scale_bits, void* feat_a, void* feat_b,
             double* pair_norm, float* ctf_out, float* spectrum_out, bool write_signed,
             cudaStream_t s);
int avg_store(const mem_plan& P, const float* avg_real, double* img_avg, double* img_avg_flip,
              const uint8_t* pd_mask, cudaStream_t s);
int intensity(const mem_plan& P, const float* flip_imgs, const PdDev* pds, double* out,
              cudaStream_t s);

// ---- D contraction (gemm_fp32.cu / gemm_tc.cu) ----------------------------------------
int gemm_fp32(const mem_plan& P, const float* feat, const double* pair_norm,
              const uint32_t* scale_bits, const Tile* tiles, const PdDev* pds,
              const int4* chunks, double* D, cudaStream_t s);
int gemm_split_bf16(const mem_plan& P, const void* feat_hi, const void* feat_lo,
                    const double* pair_norm, const uint32_t* scale_bits, const Tile* tiles,
                    const PdDev* pds, const int4* chunks, double* D, uint32_t* status,
                    cudaStream_t s);
}  // namespace kern

std::vector<int32_t> radius_descending_columns(int N, int64_t Kc, int64_t Kc_pad);

// default contraction schedule: one class, one CTA per 128 x 128 tile, two TMEM accumulators
// (MEM_TC_PERSISTENT / MEM_TC_BUFS / MEM_TC_TILE_N override it, for tuning)
mem_contraction_config default_contraction();

// orders the plan's tiles by size class and sets tc_classes / tc_ranges
int apply_contraction(mem_plan* P, int n_classes, const mem_contraction_config* classes);

// largest half-plane size for ring features (the features kernel keeps one float per frequency
// in shared memory); larger boxes use per-frequency U', V' blocks
constexpr int64_t kRingMaxKc = 40960;

// sets Kc_pad, colmap, the ring tables, Kr, Kr_pad, Kf and the chunk schedule of a plan whose N,
// Nh, Kc and ring_features are set
void feature_layout(mem_plan* P);

// device pointers of the feature tables uploaded at `base` (P.ftab copied there)
inline FeatTables feat_tables(const mem_plan& P, const void* base) {
    const int32_t* w = static_cast<const int32_t*>(base);
    return FeatTables{w, w + P.ft_ring_start, w + P.ft_ring_m, w + P.ft_pos_of, w + P.ft_ring_of,
                      reinterpret_cast<const int4*>(w + P.ft_chunks)};
}

// per-PD centring vectors: means[pd * means_stride + b * Kc_pad + k], blocks b = u, v, r, s;
// with ring features a fifth block [Kr_pad] holds the ring means of C^2 (mt)
inline int64_t means_stride(const mem_plan& P) {
    return 4 * P.Kc_pad + (P.ring_features ? P.Kr_pad : 0);
}

// power-of-two feature scale of a PD from the bit pattern of its largest |mean| (host+device)
__host__ __device__ inline float feature_scale_from_bits(uint32_t bits) {
    union { uint32_t u; float f; } cv;
    cv.u = bits;
    const float mx = cv.f;
    if (!(mx > 0.f) || mx > 3.0e38f) return 1.0f;
    const int e = (int)((bits >> 23) & 0xff) - 126;   // mx = m * 2^e, m in [0.5, 1)
    return ldexpf(1.0f, -e);
}

}  // namespace mem

#define MEM_CUDA_TRY(expr)                                    \
    do {                                                      \
        cudaError_t _e = (expr);                              \
        if (_e != cudaSuccess) return MEM_ERR_CUDA;           \
    } while (0)

#define MEM_LAUNCH_CHECK()                                    \
    do {                                                      \
        cudaError_t _e = cudaGetLastError();                  \
        if (_e != cudaSuccess) return MEM_ERR_CUDA;           \
    } while (0)
