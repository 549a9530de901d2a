// mem_pd_distances_noalloc: the distance matrix of one PD from its spectra, for callers that
// cannot allocate device memory.
//
// Some callers of this library cannot call cudaMalloc or hand us a workspace: code that runs
// while the application's allocator is locked or owned by another runtime (a host program that
// gives plugins device pointers to its own buffers but no allocation rights), code invoked from
// a memory-pool callback, or code that must not add allocation latency or fragmentation on a
// latency-critical path.  For them this entry point keeps all of its scratch in one file-scope
// static device array of MEM_NOALLOC_SCRATCH_BYTES (held by every GPU that loads the library
// until the process exits) and makes no cudaMalloc, cudaFree, cuFFT-plan or other allocating
// call.  It runs the same kernels as mem_plan_execute's CTF sums, centring, features and
// contraction, on one PD, starting from the PD's half-plane spectra (no FFT, which would need a
// cuFFT plan).
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <mutex>
#include <vector>

#include "mem_internal.cuh"

namespace mem {
namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[MEM_NOALLOC_SCRATCH_BYTES];

// per device: the scratch array's device address and the SM count, resolved once (first call on
// the device, with the device current); the feature-layout tables resident in the array (box
// size and ring setting of the copy there, -1 = none)
constexpr int kMaxDevices = 64;
struct DeviceSlot {
    std::once_flag once;
    int err = cudaSuccess;
    void* ptr = nullptr;
    int sms = 0;
    std::mutex mu;              // guards the resident-table record
    long long ftab_key = -1;
};
DeviceSlot g_slot[kMaxDevices];

int resolve_device(int dev, DeviceSlot** out) {
    DeviceSlot& d = g_slot[dev];
    std::call_once(d.once, [&d, dev]() {
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        int sms = 0;
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        d.err = (int)e;
        d.ptr = ptr;
        d.sms = sms;
    });
    if (d.err != cudaSuccess || !d.ptr) return MEM_ERR_CUDA;
    *out = &d;
    return MEM_OK;
}

size_t a256(size_t x) { return (x + 255) / 256 * 256; }

// The array's layout: the status word, the feature-layout tables (a function of the box size
// only, at a fixed offset so that a copy stays valid for later calls with the same box size),
// then the per-call tables and buffers.
struct NoallocLayout {
    size_t status, colmap, pd_table, items, item_off, img_pd, img_row, tiles, qfix, partial, means,
        avg_spec, pd_max, spec, feat_a, feat_b, pair_norm, total;
};

NoallocLayout layout_for(const mem_plan& P) {
    NoallocLayout L{};
    size_t off = 0;
    auto take = [&](size_t b) {
        const size_t o = off;
        off = a256(off + std::max<size_t>(b, 1));
        return o;
    };
    const size_t feat_elem = (P.params.precision == MEM_PREC_FP32) ? 4 : 2;
    L.status = take(16);
    L.colmap = take(sizeof(int32_t) * P.ftab.size());
    L.pd_table = take(sizeof(PdDev));
    L.items = take(sizeof(SumItem) * P.items.size());
    L.item_off = take(sizeof(int32_t) * 2);
    L.img_pd = take(sizeof(int32_t) * P.n_images);
    L.img_row = take(sizeof(int32_t) * P.n_images);
    L.tiles = take(sizeof(Tile) * P.tiles.size());
    L.qfix = take(sizeof(uint64_t) * P.n_images);
    L.partial = take(sizeof(float) * 6 * P.Kc * P.items.size());
    L.means = take(sizeof(float) * means_stride(P));
    L.avg_spec = take(sizeof(float) * 4 * P.Kc);
    L.pd_max = take(sizeof(uint32_t));
    L.spec = take(sizeof(float) * 2 * P.Kc * P.n_images);
    L.feat_a = take(feat_elem * P.Kf * P.n_rows);
    L.feat_b = (feat_elem == 4) ? L.feat_a : take(feat_elem * P.Kf * P.n_rows);
    L.pair_norm = take(sizeof(double) * P.n_images);
    L.total = off;
    return L;
}

// FNV-1a hash of the feature-layout tables: identifies the copy resident in the array
long long ftab_hash(const std::vector<int32_t>& t) {
    uint64_t h = 1469598103934665603ull;
    for (int32_t v : t) {
        h ^= (uint32_t)v;
        h *= 1099511628211ull;
    }
    return (long long)(h & 0x7fffffffffffffffull);
}

// the per-call tables of a one-PD plan of n images, written on the device (no host copy):
// the PD, the partial-sum items of kSumChunk images, image -> (PD, feature row), and the
// upper-triangle tiles (I, J), I <= J < nb, in the host plan's order (I outer)
__global__ void noalloc_tables_kernel(PdDev* __restrict__ pd, SumItem* __restrict__ items,
                                      int32_t* __restrict__ item_off, int32_t* __restrict__ img_pd,
                                      int32_t* __restrict__ img_row, Tile* __restrict__ tiles,
                                      int n, int n_items, int nb, int n_tiles) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t == 0) {
        *pd = PdDev{0, 0, 0, n, 0, 1.0, 0.0};
        item_off[0] = 0;
        item_off[1] = n_items;
    }
    if (t < n) {
        img_pd[t] = 0;
        img_row[t] = t;
    }
    if (t < n_items)
        items[t] = SumItem{0, 0, (int64_t)t * kSumChunk,
                           min((int64_t)n, (int64_t)(t + 1) * kSumChunk)};
    if (t < n_tiles) {
        int I = 0, rem = t;
        while (rem >= nb - I) {
            rem -= nb - I;
            ++I;
        }
        tiles[t] = Tile{0, I, I + rem, 0};
    }
}

// host tables of a one-PD plan (no cuFFT plans, no device queries beyond the SM count)
void one_pd_tables(mem_plan& P, const mem_params& prm, int n) {
    P.params = prm;
    P.n_pd = 1;
    P.N = prm.N;
    P.Nh = prm.N / 2 + 1;
    P.Kc = (int64_t)P.N * P.Nh;
    if (const char* e = std::getenv("MEM_RING_FEATURES")) P.ring_features = std::atoi(e) != 0;
    feature_layout(&P);
    wait_settings_from_env(&P.wait_cycles, &P.test_withhold_chunk);
    P.count.assign(1, n);
    P.pd.assign(1, PdDev{0, 0, 0, n, 0, 1.0, 0.0});
    const int nb = (n + kRowBlock - 1) / kRowBlock;
    for (int I = 0; I < nb; ++I)
        for (int J = I; J < nb; ++J) P.tiles.push_back(Tile{0, I, J, 0});
    // the tile table is written by noalloc_tables_kernel: 128-wide tiles
    mem_contraction_config dc = default_contraction();
    dc.tile_n = 128;
    dc.tile_m = 128;
    apply_contraction(&P, 1, &dc);
    for (int64_t b = 0; b < n; b += kSumChunk)
        P.items.push_back(SumItem{0, 0, b, std::min<int64_t>(n, b + kSumChunk)});
    for (int k = 0; k < n; ++k) {
        P.img_pd.push_back(0);
        P.img_row.push_back(k);
    }
    P.n_images = n;
    P.n_rows = (int64_t)nb * kRowBlock;
    P.d_elems = (int64_t)n * n;
    P.n_pairs = (int64_t)n * (n - 1) / 2;
    const double lam = 12.3986 / std::sqrt((2 * 511.0 + prm.EkV) * prm.EkV);
    const double Npix = (double)P.N * prm.pix_size;
    auto fix = [](double x) -> uint64_t {
        const double v = std::ldexp(x - std::floor(x), 64);
        return v >= 18446744073709551615.0 ? 0ull : (uint64_t)v;
    };
    P.ctf.p_fix = fix(prm.Cs * 1.0e7 * lam * lam * lam / (4.0 * Npix * Npix * Npix * Npix));
    P.ctf.d_fix = fix(std::atan(prm.AmpContrast) / (2.0 * M_PI));
    P.ctf.q_scale = lam / (2.0 * Npix * Npix);
    P.ctf.amp = (float)std::sqrt(1.0 + prm.AmpContrast * prm.AmpContrast);
    if (std::isinf(prm.gaussEnv) || prm.gaussEnv <= 0.0) {
        P.ctf.env_c = 0.0f;
    } else {
        const double sigm = prm.gaussEnv / std::sqrt(2.0 * std::log(2.0));
        P.ctf.env_c = (float)(1.0 / (Npix * Npix * 2.0 * sigm * sigm));
    }
}

template <class T>
T* at(void* base, size_t off) {
    return reinterpret_cast<T*>(static_cast<char*>(base) + off);
}

}  // namespace
}  // namespace mem

using namespace mem;

extern "C" int mem_pd_distances_noalloc(const mem_params* params, int32_t n, const float* spectra,
                                        const double* df, double* D, void* stream) {
    if (!params || !spectra || !df || !D || n < 1) return MEM_ERR_INVALID;
    if (params->N < 8) return MEM_ERR_INVALID;
    if (params->N > kMaxN) return MEM_ERR_UNSUPPORTED;
    if (params->precision != MEM_PREC_FP32 && params->precision != MEM_PREC_SPLIT_BF16)
        return MEM_ERR_INVALID;
    mem_plan P;
    one_pd_tables(P, *params, n);
    const NoallocLayout L = layout_for(P);
    if (L.total > (size_t)MEM_NOALLOC_SCRATCH_BYTES) return MEM_ERR_TOO_LARGE;
    int dev = -1;
    MEM_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return MEM_ERR_INVALID;
    DeviceSlot* slot = nullptr;
    int st = resolve_device(dev, &slot);
    if (st != MEM_OK) return st;
    P.device = dev;
    P.num_sms = slot->sms;
    void* ws = slot->ptr;
    cudaStream_t s = (cudaStream_t)stream;

    MEM_CUDA_TRY(cudaMemsetAsync(at<char>(ws, L.status), 0, 16, s));
    {
        // the feature-layout tables: copied from the host only when the array holds another
        // box size's (first call on the device or a change of box size)
        std::lock_guard<std::mutex> lk(slot->mu);
        const long long key = ftab_hash(P.ftab);
        if (slot->ftab_key != key) {
            MEM_CUDA_TRY(cudaMemcpyAsync(at<char>(ws, L.colmap), P.ftab.data(),
                                         sizeof(int32_t) * P.ftab.size(), cudaMemcpyHostToDevice,
                                         s));
            slot->ftab_key = key;
        }
    }
    const int nb = (n + kRowBlock - 1) / kRowBlock;
    const int n_items = (int)P.items.size(), n_tiles = (int)P.tiles.size();
    const int fill = std::max(n, std::max(n_items, n_tiles));
    noalloc_tables_kernel<<<(fill + 255) / 256, 256, 0, s>>>(
        at<PdDev>(ws, L.pd_table), at<SumItem>(ws, L.items), at<int32_t>(ws, L.item_off),
        at<int32_t>(ws, L.img_pd), at<int32_t>(ws, L.img_row), at<Tile>(ws, L.tiles), n, n_items,
        nb, n_tiles);
    MEM_LAUNCH_CHECK();
    // the feature kernel overwrites its spectrum with sign(C) F: work on a copy in the scratch
    MEM_CUDA_TRY(cudaMemcpyAsync(at<char>(ws, L.spec), spectra, sizeof(float) * 2 * P.Kc * n,
                                 cudaMemcpyDeviceToDevice, s));
    // padding rows of the feature matrices must read as zero; the scratch keeps old contents
    const size_t feat_elem = (P.params.precision == MEM_PREC_FP32) ? 4 : 2;
    const size_t row_bytes = feat_elem * P.Kf;
    const size_t pad_rows = (size_t)(P.n_rows - n);
    if (pad_rows) {
        MEM_CUDA_TRY(cudaMemsetAsync(at<char>(ws, L.feat_a) + n * row_bytes, 0, pad_rows * row_bytes, s));
        if (L.feat_b != L.feat_a)
            MEM_CUDA_TRY(cudaMemsetAsync(at<char>(ws, L.feat_b) + n * row_bytes, 0,
                                         pad_rows * row_bytes, s));
    }
    mem_inputs in{};
    in.df = df;
#define NA_STEP(x)                   \
    do {                             \
        st = (x);                    \
        if (st != MEM_OK) return st; \
    } while (0)
    const PdDev* pds = at<PdDev>(ws, L.pd_table);
    float2* spec = at<float2>(ws, L.spec);
    uint64_t* qf = at<uint64_t>(ws, L.qfix);
    uint32_t* pd_max = at<uint32_t>(ws, L.pd_max);
    const uint32_t* scale_bits = pd_max;
    float* means = at<float>(ws, L.means);
    double* pair_norm = at<double>(ws, L.pair_norm);
    NA_STEP(kern::qfix(P, in, qf, s));
    NA_STEP(kern::pd_sums(P, spec, qf, at<SumItem>(ws, L.items), at<float>(ws, L.partial), 3, s));
    const FeatTables ft = feat_tables(P, at<char>(ws, L.colmap));
    NA_STEP(kern::pd_finalize(P, at<float>(ws, L.partial), at<SumItem>(ws, L.items),
                              at<int32_t>(ws, L.item_off), pds, ft.ring_of, means,
                              at<float2>(ws, L.avg_spec), pd_max, 3, s));
    NA_STEP(kern::features(P, spec, qf, pds, at<int32_t>(ws, L.img_pd), at<int32_t>(ws, L.img_row),
                           ft, means, scale_bits, at<char>(ws, L.feat_a),
                           at<char>(ws, L.feat_b), pair_norm, nullptr, nullptr, false, s));
    if (P.params.precision == MEM_PREC_FP32)
        NA_STEP(kern::gemm_fp32(P, at<float>(ws, L.feat_a), pair_norm, scale_bits,
                                at<Tile>(ws, L.tiles), pds, ft.chunks, D, s));
    else
        NA_STEP(kern::gemm_split_bf16(P, at<char>(ws, L.feat_a), at<char>(ws, L.feat_b),
                                      pair_norm, scale_bits, at<Tile>(ws, L.tiles), pds,
                                      ft.chunks, D, at<uint32_t>(ws, L.status), s));
#undef NA_STEP
    return MEM_OK;
}

extern "C" int mem_noalloc_status(void* stream) {
    int dev = -1;
    MEM_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return MEM_ERR_INVALID;
    DeviceSlot* slot = nullptr;
    const int st = resolve_device(dev, &slot);
    if (st != MEM_OK) return st;
    MEM_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
    uint32_t word = 0;
    MEM_CUDA_TRY(cudaMemcpy(&word, slot->ptr, sizeof(word), cudaMemcpyDeviceToHost));
    if (word & kStatusTimeout) return MEM_ERR_DEVICE_TIMEOUT;
    return MEM_OK;
}
