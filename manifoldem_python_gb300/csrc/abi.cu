// C ABI of the distance stage: plans, workspace layout, cuFFT plan cache and the per-call
// pipeline.  See include/manifoldem_gb300.h for the contract.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <tuple>

#include "mem_internal.cuh"

namespace mem {
namespace {

constexpr size_t kAlign = 256;
inline size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

// ---- cuFFT plan cache: (N, kind, batch) -> plan, work size ----------------------------
struct FftPlan {
    cufftHandle h = 0;
    size_t work = 0;
};
std::mutex g_fft_mu;
std::map<std::tuple<int, int, int, int>, FftPlan> g_fft;   // (device, N, kind, batch)

int fft_plan(int device, int N, cufftType type, int batch, FftPlan* out) {
    std::lock_guard<std::mutex> lk(g_fft_mu);
    auto key = std::make_tuple(device, N, (int)type, batch);
    auto it = g_fft.find(key);
    if (it != g_fft.end()) {
        *out = it->second;
        return MEM_OK;
    }
    FftPlan p;
    if (cufftCreate(&p.h) != CUFFT_SUCCESS) return MEM_ERR_CUFFT;
    if (cufftSetAutoAllocation(p.h, 0) != CUFFT_SUCCESS) return MEM_ERR_CUFFT;
    int n[2] = {N, N};
    const int Nh = N / 2 + 1;
    cufftResult r;
    if (type == CUFFT_R2C)
        r = cufftMakePlanMany(p.h, 2, n, nullptr, 1, N * N, nullptr, 1, N * Nh, type, batch,
                              &p.work);
    else
        r = cufftMakePlanMany(p.h, 2, n, nullptr, 1, N * Nh, nullptr, 1, N * N, type, batch,
                              &p.work);
    if (r != CUFFT_SUCCESS) {
        cufftDestroy(p.h);
        return MEM_ERR_CUFFT;
    }
    g_fft[key] = p;
    *out = p;
    return MEM_OK;
}

size_t fft_work_estimate(int N, cufftType type, int batch) {
    int n[2] = {N, N};
    const int Nh = N / 2 + 1;
    size_t ws = 0;
    cufftResult r = type == CUFFT_R2C
        ? cufftEstimateMany(2, n, nullptr, 1, N * N, nullptr, 1, N * Nh, type, batch, &ws)
        : cufftEstimateMany(2, n, nullptr, 1, N * Nh, nullptr, 1, N * N, type, batch, &ws);
    return r == CUFFT_SUCCESS ? ws : 0;
}

// batch sizes exec_fft uses for `count` transforms: full chunks and the remainder
void fft_batches(int64_t count, std::vector<int>* batches) {
    if (count >= kFftChunk) batches->push_back(kFftChunk);
    if (count % kFftChunk) batches->push_back((int)(count % kFftChunk));
}

}  // namespace

size_t fft_work_bytes(int N, cufftType type, int64_t count) {
    std::vector<int> batches;
    fft_batches(count, &batches);
    size_t work = 0;
    for (int b : batches) work = std::max(work, fft_work_estimate(N, type, b));
    return work;
}

int fft_exec(int device, int N, cufftType type, int64_t count, int64_t in_stride,
             int64_t out_stride, void* in, void* out, void* work, cudaStream_t s) {
    for (int64_t b = 0; b < count; b += kFftChunk) {
        const int batch = (int)std::min<int64_t>(kFftChunk, count - b);
        FftPlan fp;
        int st = fft_plan(device, N, type, batch, &fp);
        if (st != MEM_OK) return st;
        if (cufftSetStream(fp.h, s) != CUFFT_SUCCESS) return MEM_ERR_CUFFT;
        if (cufftSetWorkArea(fp.h, work) != CUFFT_SUCCESS) return MEM_ERR_CUFFT;
        cufftResult r;
        if (type == CUFFT_R2C)
            r = cufftExecR2C(fp.h, (cufftReal*)in + b * in_stride,
                             (cufftComplex*)out + b * out_stride);
        else
            r = cufftExecC2R(fp.h, (cufftComplex*)in + b * in_stride,
                             (cufftReal*)out + b * out_stride);
        if (r != CUFFT_SUCCESS) return MEM_ERR_CUFFT;
    }
    return MEM_OK;
}

namespace {

int exec_fft(const mem_plan& P, cufftType type, int64_t count, int64_t in_stride,
             int64_t out_stride, void* in, void* out, void* work, cudaStream_t s) {
    return fft_exec(P.device, P.N, type, count, in_stride, out_stride, in, out, work, s);
}

template <class T>
T* at(void* ws, size_t off) {
    return reinterpret_cast<T*>(static_cast<char*>(ws) + off);
}

}  // namespace
// feature column of each frequency slot k in [0, Kc_pad) (k >= Kc are zero padding): whole
// 64-wide chunks of consecutive k are reordered by decreasing smallest |k|^2 in the chunk, so the
// chunks holding the dominant low frequencies are accumulated last, while the columns inside a
// chunk stay in natural order (coalesced feature stores).
std::vector<int32_t> radius_descending_columns(int N, int64_t Kc, int64_t Kc_pad) {
    const int Nh = N / 2 + 1;
    const int64_t nch = Kc_pad / kKPad;
    std::vector<int64_t> key(nch, INT64_MAX);
    for (int64_t k = 0; k < Kc; ++k) {
        const int ka = (int)(k / Nh), kb = (int)(k % Nh);
        const int fa = std::min(ka, N - ka);
        key[k / kKPad] = std::min<int64_t>(key[k / kKPad], (int64_t)fa * fa + (int64_t)kb * kb);
    }
    std::vector<int32_t> order(nch);
    for (int64_t c = 0; c < nch; ++c) order[c] = (int32_t)c;
    std::stable_sort(order.begin(), order.end(),
                     [&](int32_t a, int32_t b) { return key[a] > key[b]; });
    std::vector<int32_t> pos(nch);
    for (int64_t r = 0; r < nch; ++r) pos[order[r]] = (int32_t)r;
    std::vector<int32_t> col(Kc_pad);
    for (int64_t k = 0; k < Kc_pad; ++k) col[k] = (int32_t)(pos[k / kKPad] * kKPad + k % kKPad);
    return col;
}

// Feature layout.  Ring features: the C^2 |F|^2 part of D, sum_k w C_j(k)^2 |F_i(k)|^2, depends on
// the CTF only through |k|^2 (C is radial), so it is a sum over rings of equal |k|^2 of
// C_j(ring)^2 times the ring sums of w |F_i|^2: U', V' get one column per ring instead of one per
// frequency (1621 rings for 8320 half-plane frequencies at 128 px).  Rings are ordered by
// decreasing |k|^2, members within a ring by k.  The contraction's K chunks interleave the
// (U', V') and (r', s') chunk pairs in proportion, so that the low frequencies of both come last.
void feature_layout(mem_plan* P) {
    const int N = P->N, Nh = P->Nh;
    const int64_t Kc = P->Kc;
    P->Kc_pad = (Kc + kKPad - 1) / kKPad * kKPad;
    P->colmap = radius_descending_columns(N, Kc, P->Kc_pad);
    P->ring_features = P->ring_features && Kc <= kRingMaxKc;
    std::vector<int32_t> ring_start, ring_m, pos_of, ring_of;
    if (P->ring_features) {
        std::vector<int64_t> mk(Kc);
        std::vector<int32_t> order(Kc);
        for (int64_t k = 0; k < Kc; ++k) {
            const int ka = (int)(k / Nh), kb = (int)(k % Nh);
            const int fa = std::min(ka, N - ka);
            mk[k] = (int64_t)fa * fa + (int64_t)kb * kb;
            order[k] = (int32_t)k;
        }
        std::stable_sort(order.begin(), order.end(),
                         [&](int32_t a, int32_t b) { return mk[a] > mk[b]; });
        pos_of.resize(Kc);
        ring_of.resize(Kc);
        for (int64_t i = 0; i < Kc; ++i) {
            if (i == 0 || mk[order[i]] != mk[order[i - 1]]) {
                ring_start.push_back((int32_t)i);
                ring_m.push_back((int32_t)mk[order[i]]);
            }
            pos_of[order[i]] = (int32_t)i;
            ring_of[order[i]] = (int32_t)ring_m.size() - 1;
        }
        ring_start.push_back((int32_t)Kc);
        P->Kr = (int64_t)ring_m.size();
        P->Kr_pad = (P->Kr + kKPad - 1) / kKPad * kKPad;
    } else {
        ring_start.push_back(0);
        P->Kr = Kc;
        P->Kr_pad = P->Kc_pad;
    }
    P->Kf = 2 * P->Kr_pad + 2 * P->Kc_pad;
    const int64_t Kr_pad = P->Kr_pad, Kc_pad = P->Kc_pad;
    std::vector<int4> ch;
    const int64_t nu = Kr_pad / kKPad, nr = Kc_pad / kKPad;
    // w = 1: the split-BF16 contraction adds the lo.lo product for the chunk.  Ring sums are
    // fewer and larger terms than per-frequency products, so their split error weighs more; the
    // largest are the low-frequency rings of the last 4 (U', V') chunk pairs
    // (MEM_RING_LOLO_PAIRS overrides the count, for tuning)
    int64_t lolo_pairs = 4;
    if (const char* e = std::getenv("MEM_RING_LOLO_PAIRS")) lolo_pairs = std::atoll(e);
    auto push_uv = [&](int64_t q) {
        const int lolo = (P->ring_features && q >= nu - lolo_pairs) ? 1 : 0;
        ch.push_back(make_int4((int)(q * kKPad), (int)(Kr_pad + q * kKPad), 0, lolo));
        ch.push_back(make_int4((int)(Kr_pad + q * kKPad), (int)(q * kKPad), 0, lolo));
    };
    auto push_rs = [&](int64_t q) {
        const int a = (int)(2 * Kr_pad + q * kKPad), b = (int)(2 * Kr_pad + Kc_pad + q * kKPad);
        ch.push_back(make_int4(a, a, 1, 0));
        ch.push_back(make_int4(b, b, 1, 0));
    };
    if (!P->ring_features) {
        for (int64_t q = 0; q < nr; ++q) {      // u', v', r', s' chunk q in turn
            push_uv(q);
            push_rs(q);
        }
    } else {
        int64_t i = 0, j = 0;
        while (i < nu || j < nr) {
            if (j >= nr || (i < nu && (2 * i + 1) * nr <= (2 * j + 1) * nu))
                push_uv(i++);
            else
                push_rs(j++);
        }
    }
    P->n_chunks = (int)ch.size();
    // one int32 table: colmap | ring_start | ring_m | pos_of | ring_of | chunks (16-byte aligned)
    std::vector<int32_t>& t = P->ftab;
    t.assign(P->colmap.begin(), P->colmap.end());
    P->ft_ring_start = t.size();
    t.insert(t.end(), ring_start.begin(), ring_start.end());
    P->ft_ring_m = t.size();
    t.insert(t.end(), ring_m.begin(), ring_m.end());
    P->ft_pos_of = t.size();
    t.insert(t.end(), pos_of.begin(), pos_of.end());
    P->ft_ring_of = t.size();
    t.insert(t.end(), ring_of.begin(), ring_of.end());
    while (t.size() % 4) t.push_back(0);
    P->ft_chunks = t.size();
    for (const int4& c : ch) {
        t.push_back(c.x);
        t.push_back(c.y);
        t.push_back(c.z);
        t.push_back(c.w);
    }
}
namespace {

CtfConst make_ctf(const mem_params& p, int N) {
    CtfConst c{};
    const double lam = 12.3986 / std::sqrt((2 * 511.0 + p.EkV) * p.EkV);
    const double Npix = (double)N * p.pix_size;
    const double P = p.Cs * 1.0e7 * lam * lam * lam / (4.0 * Npix * Npix * Npix * Npix);
    const double d = std::atan(p.AmpContrast) / (2.0 * M_PI);
    auto fix = [](double x) -> uint64_t {
        double fr = x - std::floor(x);
        double v = std::ldexp(fr, 64);
        if (v >= 18446744073709551615.0) return 0ull;
        return (uint64_t)v;
    };
    c.p_fix = fix(P);
    c.d_fix = fix(d);
    c.q_scale = lam / (2.0 * Npix * Npix);
    c.amp = (float)std::sqrt(1.0 + p.AmpContrast * p.AmpContrast);
    if (std::isinf(p.gaussEnv) || p.gaussEnv <= 0.0) {
        c.env_c = 0.0f;
    } else {
        const double sigm = p.gaussEnv / std::sqrt(2.0 * std::log(2.0));
        c.env_c = (float)(1.0 / (Npix * Npix * 2.0 * sigm * sigm));
    }
    return c;
}

}  // namespace

void wait_settings_from_env(long long* cycles, int* withhold) {
    *cycles = kDefaultWaitCycles;
    *withhold = -1;
    if (const char* e = std::getenv("MEM_WAIT_CYCLES")) {
        const long long v = std::atoll(e);
        if (v >= 1000) *cycles = v;
    }
    if (const char* e = std::getenv("MEM_TEST_WITHHOLD_CHUNK")) *withhold = std::atoi(e);
}

mem_contraction_config default_contraction() {
    mem_contraction_config c{INT32_MAX, 0, 2, 128, 128, 0};
    if (const char* e = std::getenv("MEM_TC_PERSISTENT")) c.persistent = std::atoi(e) != 0;
    if (const char* e = std::getenv("MEM_TC_BUFS")) c.accumulators = std::atoi(e) == 4 ? 4 : 2;
    if (const char* e = std::getenv("MEM_TC_TILE_N")) c.tile_n = std::atoi(e) == 256 ? 256 : 128;
    if (const char* e = std::getenv("MEM_TC_TILE_M")) c.tile_m = std::atoi(e) == 256 ? 256 : 128;
    if (c.tile_n == 256) c.accumulators = 2;
    if (c.tile_m == 256) c.tile_n = 128;
    return c;
}

int apply_contraction(mem_plan* P, int n_classes, const mem_contraction_config* classes) {
    if (n_classes < 1 || !classes) return MEM_ERR_INVALID;
    for (int k = 0; k < n_classes; ++k) {
        const mem_contraction_config& c = classes[k];
        if (c.max_n < 1 || (k > 0 && c.max_n <= classes[k - 1].max_n)) return MEM_ERR_INVALID;
        if (c.persistent != 0 && c.persistent != 1) return MEM_ERR_INVALID;
        if (c.accumulators != 2 && c.accumulators != 4) return MEM_ERR_INVALID;
        if (c.tile_n != 0 && c.tile_n != 128 && c.tile_n != 256) return MEM_ERR_INVALID;
        if (c.tile_m != 0 && c.tile_m != 128 && c.tile_m != 256) return MEM_ERR_INVALID;
        if (c.tile_n == 256 && c.accumulators != 2) return MEM_ERR_INVALID;
        if (c.tile_m == 256 && c.tile_n == 256) return MEM_ERR_INVALID;
    }
    auto cls = [&](int n) {
        for (int k = 0; k < n_classes - 1; ++k)
            if (n <= classes[k].max_n) return k;
        return n_classes - 1;
    };
    P->tc_classes.assign(classes, classes + n_classes);
    for (mem_contraction_config& c : P->tc_classes) {
        // the compensated epilogue sums (a tuning option) exist in the one-SM 128 x 128 kernel
        // only: the 256-wide tile's would not fit the register file
        if (c.tile_n != 256 || P->tc_kahan) c.tile_n = 128;
        if (c.tile_m != 256 || P->tc_kahan) c.tile_m = 128;
    }
    // the tiles of every class, class by class, PDs in plan order: row blocks I and column
    // blocks J of the class's tile shape that meet the upper triangle (J >= I bm / bn)
    P->tc_tiles.clear();
    P->tc_ranges.assign(n_classes, std::make_pair(0, 0));
    for (int k = 0; k < n_classes; ++k) {
        const int bn = P->tc_classes[k].tile_n, bm = P->tc_classes[k].tile_m;
        P->tc_ranges[k].first = (int)P->tc_tiles.size();
        for (int i = 0; i < P->n_pd; ++i) {
            const int n = P->pd[i].n;
            if (cls(n) != k) continue;
            const int nb = (n + bm - 1) / bm, nj = (n + bn - 1) / bn;
            for (int I = 0; I < nb; ++I)
                for (int J = (I * bm) / bn; J < nj; ++J)
                    P->tc_tiles.push_back(Tile{i, I, J, 0});
        }
        P->tc_ranges[k].second = (int)P->tc_tiles.size() - P->tc_ranges[k].first;
    }
    return MEM_OK;
}

namespace {

int check_device(int* device, int* sms) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return MEM_ERR_NO_DEVICE;
    }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) return MEM_ERR_CUDA;
    *device = dev;
    *sms = prop.multiProcessorCount;
    return MEM_OK;
}

}  // namespace
}  // namespace mem

using namespace mem;

extern "C" {

int mem_abi_version(void) { return MEM_ABI_VERSION; }

const char* mem_status_string(int status) {
    switch (status) {
        case MEM_OK: return "ok";
        case MEM_ERR_INVALID: return "invalid argument";
        case MEM_ERR_UNSUPPORTED: return "unsupported box size or option";
        case MEM_ERR_WORKSPACE: return "workspace too small";
        case MEM_ERR_CUDA: return "CUDA runtime error";
        case MEM_ERR_CUFFT: return "cuFFT error";
        case MEM_ERR_DEVICE_TIMEOUT: return "bounded device-side wait expired";
        case MEM_ERR_NO_DEVICE: return "no CUDA device";
        case MEM_ERR_TOO_LARGE: return "too large for the no-allocation entry point's static scratch";
        default: return "unknown status";
    }
}

int mem_plan_create(const mem_params* params, int32_t n_pd, const int32_t* pd_count,
                    const double* psi_p_deg, mem_plan** out_plan) {
    if (!params || !pd_count || !psi_p_deg || !out_plan || n_pd < 1) return MEM_ERR_INVALID;
    *out_plan = nullptr;
    const mem_params& p = *params;
    if (p.N < 8) return MEM_ERR_INVALID;
    if (p.N > kMaxN) return MEM_ERR_UNSUPPORTED;
    if (p.filter_type != MEM_FILTER_BUTTER && p.filter_type != MEM_FILTER_GAUSS)
        return MEM_ERR_INVALID;
    if (p.precision != MEM_PREC_FP32 && p.precision != MEM_PREC_SPLIT_BF16)
        return MEM_ERR_INVALID;
    if (!(p.pix_size > 0) || !(p.EkV > 0) || !(p.filter_Qc > 0)) return MEM_ERR_INVALID;
    for (int i = 0; i < n_pd; ++i) {
        if (pd_count[i] < 1) return MEM_ERR_INVALID;
        if (!std::isfinite(psi_p_deg[i])) return MEM_ERR_INVALID;
    }
    mem_plan* P = new (std::nothrow) mem_plan();
    if (!P) return MEM_ERR_INVALID;
    P->params = p;
    P->n_pd = n_pd;
    P->N = p.N;
    P->Nh = p.N / 2 + 1;
    P->Kc = (int64_t)P->N * P->Nh;
    // ring features for the U', V' blocks (MEM_RING_FEATURES=0 selects per-frequency blocks)
    if (const char* e = std::getenv("MEM_RING_FEATURES")) P->ring_features = std::atoi(e) != 0;
    feature_layout(P);
    P->count.assign(pd_count, pd_count + n_pd);
    P->pd.resize(n_pd);
    int64_t img = 0, row = 0, d = 0, pairs = 0;
    for (int i = 0; i < n_pd; ++i) {
        const int n = pd_count[i];
        PdDev& q = P->pd[i];
        q.img_off = img;
        q.row_off = row;
        q.d_off = d;
        q.n = n;
        q.pad = 0;
        const double t = (-psi_p_deg[i]) * (M_PI / 180.0);
        q.rot2_cos = std::cos(t);
        q.rot2_sin = std::sin(t);
        const int nb = (n + kRowBlock - 1) / kRowBlock;
        for (int I = 0; I < nb; ++I)
            for (int J = I; J < nb; ++J) P->tiles.push_back(Tile{i, I, J, 0});
        for (int64_t b = 0; b < n; b += kSumChunk)
            P->items.push_back(SumItem{i, 0, img + b, img + std::min<int64_t>(n, b + kSumChunk)});
        for (int k = 0; k < n; ++k) {
            P->img_pd.push_back(i);
            P->img_row.push_back((int32_t)(row + k));
        }
        img += n;
        row += (int64_t)nb * kRowBlock;
        d += (int64_t)n * n;
        pairs += (int64_t)n * (n - 1) / 2;
    }
    P->n_images = img;
    P->n_rows = row;
    P->d_elems = d;
    P->n_pairs = pairs;
    if (row > INT32_MAX) {
        delete P;
        return MEM_ERR_UNSUPPORTED;
    }
    P->ctf = make_ctf(p, P->N);
    // tensor-core accumulation knobs (tuning; the defaults are the validated setting)
    if (const char* e = std::getenv("MEM_TC_GROUP_CHUNKS")) P->tc_group_chunks = std::atoi(e);
    if (const char* e = std::getenv("MEM_TC_KAHAN")) P->tc_kahan = std::atoi(e) != 0;
    if (const char* e = std::getenv("MEM_TC_TERMS")) P->tc_lolo = std::atoi(e) >= 4;
    {
        const mem_contraction_config dc = default_contraction();
        apply_contraction(P, 1, &dc);
    }
    // image transforms: the shared-memory FFT kernels where they exist (MEM_SMEM_FFT=0 selects
    // cuFFT, for comparison)
    if (const char* e = std::getenv("MEM_SMEM_FFT")) P->smem_fft = std::atoi(e) != 0;
    P->smem_fft = P->smem_fft && kern::smem_fft_supported(*P);
    if (const char* e = std::getenv("MEM_FUSED_IMAGE")) P->fused_image = std::atoi(e) != 0;
    P->fused_image = P->fused_image && P->smem_fft && kern::image_stage_supported(*P);
    if (const char* e = std::getenv("MEM_ROT_BAND")) P->rot_band = std::atoi(e);
    if (const char* e = std::getenv("MEM_ROT_BAND_VARIANT"))
        P->rot_band_variant = std::min(3, std::max(0, std::atoi(e)));
    wait_settings_from_env(&P->wait_cycles, &P->test_withhold_chunk);
    if (const char* e = std::getenv("MEM_HOST_LOAD_CTAS")) P->host_load_ctas = std::atoi(e);
    if (const char* e = std::getenv("MEM_HOST_LOAD_THREADS")) {
        const int t = std::atoi(e);
        if (t == 256 || t == 512 || t == 1024) P->host_load_threads = t;
    }

    // cuFFT work sizes: exact when a device is current, an estimate otherwise
    std::vector<int> img_batches;
    fft_batches(P->n_images, &img_batches);
    fft_batches(2 * (int64_t)n_pd, &img_batches);
    const bool have_dev = check_device(&P->device, &P->num_sms) == MEM_OK;
    if (!have_dev) {
        P->device = -1;
        P->num_sms = 152;
    }
    size_t work = 0;
    if (P->smem_fft) img_batches.clear();      // no cuFFT plan is used
    for (int b : img_batches) {
        for (cufftType ty : {CUFFT_R2C, CUFFT_C2R}) {
            if (have_dev) {
                FftPlan fp;
                const int st = fft_plan(P->device, P->N, ty, b, &fp);
                if (st != MEM_OK) {
                    delete P;
                    return st;
                }
                work = std::max(work, fp.work);
            } else {
                work = std::max(work, 2 * fft_work_estimate(P->N, ty, b));
            }
        }
    }
    P->cufft_work_bytes = work;

    // workspace layout
    Layout& L = P->lay;
    const int64_t NN = (int64_t)P->N * P->N;
    const size_t feat_elem = (p.precision == MEM_PREC_FP32) ? 4 : 2;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off = align_up(off + std::max<size_t>(bytes, 1));
        return o;
    };
    L.status = take(sizeof(uint32_t) * 4);
    L.pd_table = take(sizeof(PdDev) * n_pd);
    L.sum_items = take(sizeof(SumItem) * P->items.size());
    L.item_off = take(sizeof(int32_t) * (n_pd + 1));
    L.img_pd = take(sizeof(int32_t) * P->n_images);
    L.img_row = take(sizeof(int32_t) * P->n_images);
    L.tiles = take(sizeof(Tile) * P->tiles.size());
    L.tc_tiles = take(sizeof(Tile) * P->tiles.size());   // >= the tiles of any width >= 128
    L.qfix = take(sizeof(uint64_t) * P->n_images);
    L.rotc = take(64 * (size_t)P->n_images);            // two fixed-point rotations per image
    L.gtab = take(sizeof(float) * P->N * P->Nh);
    L.pd_max = take(sizeof(uint32_t) * n_pd);
    L.colmap = take(sizeof(int32_t) * P->ftab.size());
    L.twid = take(sizeof(float) * 2 * (P->N / 2 + 1));
    L.ident = take(sizeof(int64_t) * P->n_images);      // 0..n-1: stack index of shifted copies
    L.xbuf = take(sizeof(float) * NN * P->n_images);
    L.spec = take(sizeof(float) * 2 * P->Kc * P->n_images);
    L.feat_a = take(feat_elem * P->Kf * P->n_rows);
    L.feat_b = (p.precision == MEM_PREC_FP32) ? L.feat_a : take(feat_elem * P->Kf * P->n_rows);
    L.pair_norm = take(sizeof(double) * P->n_images);
    L.partial = take(sizeof(float) * 6 * P->Kc * P->items.size());
    L.means = take(sizeof(float) * means_stride(*P) * n_pd);
    L.avg_spec = take(sizeof(float) * 2 * 2 * P->Kc * n_pd);
    L.avg_real = take(sizeof(float) * 2 * NN * n_pd);
    L.cufft_work = take(P->cufft_work_bytes);
    L.total = off;
    *out_plan = P;
    return MEM_OK;
}

int mem_plan_destroy(mem_plan* plan) {
    delete plan;
    return MEM_OK;
}

int mem_plan_workspace_size(const mem_plan* plan, size_t* bytes) {
    if (!plan || !bytes) return MEM_ERR_INVALID;
    *bytes = plan->lay.total;
    return MEM_OK;
}

int64_t mem_plan_num_images(const mem_plan* plan) { return plan ? plan->n_images : -1; }
int64_t mem_plan_d_elements(const mem_plan* plan) { return plan ? plan->d_elems : -1; }
int64_t mem_plan_num_pairs(const mem_plan* plan) { return plan ? plan->n_pairs : -1; }

int mem_plan_set_contraction(mem_plan* plan, int32_t n_classes,
                             const mem_contraction_config* classes) {
    if (!plan || plan->uploaded) return MEM_ERR_INVALID;
    return apply_contraction(plan, n_classes, classes);
}

int mem_plan_upload(mem_plan* plan, void* workspace, size_t workspace_bytes, void* stream) {
    if (!plan || !workspace) return MEM_ERR_INVALID;
    plan->uploaded = true;
    if (workspace_bytes < plan->lay.total) return MEM_ERR_WORKSPACE;
    if (plan->device < 0) {
        int st = check_device(&plan->device, &plan->num_sms);
        if (st != MEM_OK) return st;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const mem_plan& P = *plan;
    const Layout& L = P.lay;
    std::vector<int32_t> item_off(P.n_pd + 1, 0);
    for (const SumItem& it : P.items) item_off[it.pd + 1]++;
    for (int i = 0; i < P.n_pd; ++i) item_off[i + 1] += item_off[i];
    MEM_CUDA_TRY(cudaMemcpyAsync(at<char>(workspace, L.pd_table), P.pd.data(),
                                 sizeof(PdDev) * P.n_pd, cudaMemcpyHostToDevice, s));
    MEM_CUDA_TRY(cudaMemcpyAsync(at<char>(workspace, L.sum_items), P.items.data(),
                                 sizeof(SumItem) * P.items.size(), cudaMemcpyHostToDevice, s));
    MEM_CUDA_TRY(cudaMemcpyAsync(at<char>(workspace, L.item_off), item_off.data(),
                                 sizeof(int32_t) * item_off.size(), cudaMemcpyHostToDevice, s));
    MEM_CUDA_TRY(cudaMemcpyAsync(at<char>(workspace, L.img_pd), P.img_pd.data(),
                                 sizeof(int32_t) * P.n_images, cudaMemcpyHostToDevice, s));
    MEM_CUDA_TRY(cudaMemcpyAsync(at<char>(workspace, L.img_row), P.img_row.data(),
                                 sizeof(int32_t) * P.n_images, cudaMemcpyHostToDevice, s));
    MEM_CUDA_TRY(cudaMemcpyAsync(at<char>(workspace, L.tiles), P.tiles.data(),
                                 sizeof(Tile) * P.tiles.size(), cudaMemcpyHostToDevice, s));
    if (P.tc_tiles.size() > P.tiles.size()) return MEM_ERR_INVALID;
    if (!P.tc_tiles.empty())
        MEM_CUDA_TRY(cudaMemcpyAsync(at<char>(workspace, L.tc_tiles), P.tc_tiles.data(),
                                     sizeof(Tile) * P.tc_tiles.size(), cudaMemcpyHostToDevice,
                                     s));
    MEM_CUDA_TRY(cudaMemcpyAsync(at<char>(workspace, L.colmap), P.ftab.data(),
                                 sizeof(int32_t) * P.ftab.size(), cudaMemcpyHostToDevice, s));
    {
        std::vector<int64_t> ident(P.n_images);
        for (int64_t i = 0; i < P.n_images; ++i) ident[i] = i;
        MEM_CUDA_TRY(cudaMemcpyAsync(at<char>(workspace, L.ident), ident.data(),
                                     sizeof(int64_t) * ident.size(), cudaMemcpyHostToDevice, s));
    }
    // FFT twiddles exp(-2 pi i k / N), k = 0..N/2, computed in double
    std::vector<float> tw(2 * (P.N / 2 + 1));
    for (int k = 0; k <= P.N / 2; ++k) {
        const double a = -2.0 * M_PI * k / P.N;
        tw[2 * k] = (float)std::cos(a);
        tw[2 * k + 1] = (float)std::sin(a);
    }
    MEM_CUDA_TRY(cudaMemcpyAsync(at<char>(workspace, L.twid), tw.data(), sizeof(float) * tw.size(),
                                 cudaMemcpyHostToDevice, s));
    // padding rows of the feature matrices stay zero for the whole life of the workspace
    const size_t feat_elem = (P.params.precision == MEM_PREC_FP32) ? 4 : 2;
    const size_t row_bytes = feat_elem * P.Kf;
    for (int i = 0; i < P.n_pd; ++i) {
        const int n = P.pd[i].n;
        const int64_t padded = (int64_t)((n + kRowBlock - 1) / kRowBlock) * kRowBlock;
        if (padded == n) continue;
        const size_t o = (size_t)(P.pd[i].row_off + n) * row_bytes;
        const size_t len = (size_t)(padded - n) * row_bytes;
        MEM_CUDA_TRY(cudaMemsetAsync(at<char>(workspace, L.feat_a) + o, 0, len, s));
        if (L.feat_b != L.feat_a)
            MEM_CUDA_TRY(cudaMemsetAsync(at<char>(workspace, L.feat_b) + o, 0, len, s));
    }
    // the pageable sources above are consumed before cudaMemcpyAsync returns
    return MEM_OK;
}

namespace {
// true when p is host memory (pinned, registered, or pageable on a system whose GPU reads host
// page tables): the stack is then read over the host link
bool is_host_memory(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost || a.type == cudaMemoryTypeUnregistered;
}

int execute_impl(mem_plan* plan, const mem_inputs* in, const mem_outputs* out, void* workspace,
                 size_t workspace_bytes, cudaStream_t ls, cudaStream_t s);
}  // namespace

int mem_plan_execute(mem_plan* plan, const mem_inputs* in, const mem_outputs* out,
                     void* workspace, size_t workspace_bytes, void* stream) {
    return execute_impl(plan, in, out, workspace, workspace_bytes, (cudaStream_t)stream,
                        (cudaStream_t)stream);
}

int mem_plan_execute_split(mem_plan* plan, const mem_inputs* in, const mem_outputs* out,
                           void* workspace, size_t workspace_bytes, void* load_stream,
                           void* stream) {
    return execute_impl(plan, in, out, workspace, workspace_bytes, (cudaStream_t)load_stream,
                        (cudaStream_t)stream);
}

namespace {
int execute_impl(mem_plan* plan, const mem_inputs* in, const mem_outputs* out, void* workspace,
                 size_t workspace_bytes, cudaStream_t ls, cudaStream_t s) {
    if (!plan || !in || !out || !workspace) return MEM_ERR_INVALID;
    if (workspace_bytes < plan->lay.total) return MEM_ERR_WORKSPACE;
    if (!in->stack || !in->stack_index || !in->flip || !in->psi_rad || !in->df)
        return MEM_ERR_INVALID;
    if (in->num_stack < 1) return MEM_ERR_INVALID;
    if (plan->device < 0) return MEM_ERR_INVALID;   // not uploaded
    const mem_plan& P = *plan;
    const Layout& L = P.lay;
    const bool split = ls != s;
    // a split execute with the stack in host memory: the load stream only copies the entries'
    // images over the host link (a few light CTAs, so the rest of the GPU keeps computing), and
    // all the arithmetic runs on the copies on the main stream
    const bool host_copy = split && is_host_memory(in->stack);
    void* ws = workspace;
    uint32_t* status = at<uint32_t>(ws, L.status);
    mem_plan& PM = *plan;
    PM.timed_run = PM.timing;
    for (bool& r : PM.phase_ran) r = false;
    // event k marks the start of phase k; phase k ends at the next recorded event
    auto mark = [&](int phase) -> int {
        if (!PM.timing) return MEM_OK;
        MEM_CUDA_TRY(cudaEventRecord(PM.ev[phase], phase <= 2 ? ls : s));
        if (phase > 0) PM.phase_ran[phase - 1] = true;
        return MEM_OK;
    };
    const PdDev* pds = at<PdDev>(ws, L.pd_table);
    const int32_t* img_pd = at<int32_t>(ws, L.img_pd);
    const int32_t* img_row = at<int32_t>(ws, L.img_row);
    float* xbuf = at<float>(ws, L.xbuf);
    float2* spec = at<float2>(ws, L.spec);
    uint64_t* qf = at<uint64_t>(ws, L.qfix);
    void* work = at<char>(ws, L.cufft_work);
    const int64_t NN = (int64_t)P.N * P.N;
    const int64_t specN = P.Kc;
    int st;
#define MEM_STEP(x)                 \
    do {                            \
        st = (x);                   \
        if (st != MEM_OK) return st; \
    } while (0)

    // the stack is read by exactly one kernel (the first), issued on the load stream
    MEM_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(uint32_t) * 4, ls));
    MEM_STEP(mark(0));
    MEM_STEP(kern::lowpass_table(P, at<float>(ws, L.gtab), ls));
    mem_inputs lin = *in;
    const int64_t* ident = at<int64_t>(ws, L.ident);
    cudaStream_t cs = ls;                                // stream of the image arithmetic
    auto join = [&]() -> int {                           // the main stream waits for the loads
        if (!split) return MEM_OK;
        if (!PM.load_done)
            MEM_CUDA_TRY(cudaEventCreateWithFlags(&PM.load_done, cudaEventDisableTiming));
        MEM_CUDA_TRY(cudaEventRecord(PM.load_done, ls));
        MEM_CUDA_TRY(cudaStreamWaitEvent(s, PM.load_done, 0));
        return MEM_OK;
    };
    // the fused image kernel (N = 64, 128, no volume mask, SPIDER stack) writes each image's
    // spectrum while other images are still being read: its input may not sit in the spectrum
    // slots (a slot is larger than an image, so spectrum i overlaps later images' raw data)
    const bool fused = P.fused_image && !in->pd_mask && !in->shift_yx;
    if (host_copy) {
        // raw copies into free slots: xbuf when the RELION shift writes the spectrum slots or
        // the fused kernel writes them (image i's slot is read and rewritten by its own CTA
        // only), the spectrum slots otherwise
        float* staging = (in->shift_yx || fused) ? xbuf : reinterpret_cast<float*>(spec);
        MEM_STEP(kern::gather_copy(P, *in, staging, status, P.host_load_ctas, ls));
        MEM_STEP(join());
        cs = s;
        lin.stack = staging;
        lin.num_stack = P.n_images;
        lin.stack_index = ident;
    }
    if (in->shift_yx) {
        // RELION: shifted copies, laid out as SPIDER images, in the (still free) spectrum
        // slots; the gather then reads copy i for entry i
        float* shifted = reinterpret_cast<float*>(spec);
        MEM_STEP(kern::relion_shift(P, lin, shifted, status, cs));
        lin.stack = shifted;
        lin.num_stack = P.n_images;
        lin.stack_index = ident;
    }
    float* img_all = out->img_all ? out->img_all : xbuf;
    if (fused) {
        // (a2-a4, a6, a8) gather, flip, normalisation, low-pass, mask, both rotations and
        // F = fft2(imgAll) in one kernel per image; the lowpass phase holds all of it, the
        // rotate and spectrum phases are empty
        MEM_STEP(mark(1));
        MEM_STEP(kern::rot_consts(P, *in, pds, img_pd, at<char>(ws, L.rotc), cs));
        MEM_STEP(kern::image_stage(P, lin, at<float>(ws, L.gtab), at<float2>(ws, L.twid), xbuf,
                                   img_all, at<char>(ws, L.rotc), spec, status, cs));
    } else if (P.smem_fft) {
        // (a2, a3) gather, flip, normalisation and low-pass in one shared-memory pass
        MEM_STEP(mark(1));
        MEM_STEP(kern::lowpass_fused(P, lin, at<float>(ws, L.gtab), at<float2>(ws, L.twid), xbuf,
                                     status, cs));
    } else {
        // (a2) gather, conjugate flip, normalisation
        MEM_STEP(kern::gather_normalize(P, lin, xbuf, status, 0, cs));
        MEM_STEP(mark(1));
    }
    if (!host_copy) MEM_STEP(join());
    if (!P.smem_fft) {
        // (a3) low-pass filter: R2C, multiply by G/N^2, C2R
        MEM_STEP(exec_fft(P, CUFFT_R2C, P.n_images, NN, specN, xbuf, spec, work, s));
        MEM_STEP(kern::lowpass(P, spec, at<float>(ws, L.gtab), s));
        MEM_STEP(exec_fft(P, CUFFT_C2R, P.n_images, specN, NN, spec, xbuf, work, s));
    }
    MEM_STEP(mark(2));
    // (a4, a6) mask and the two rotations -> imgAll
    if (!fused)
        MEM_STEP(kern::rotate(P, *in, xbuf, img_all, pds, img_pd, spec, at<char>(ws, L.rotc), s));
    MEM_STEP(mark(3));
    // (a8) F = fft2(imgAll); (a7, a9) CTF and per-PD sums.  With a volume mask the spectra of
    // D, of the phase flips and of imgAvgFlip are those of imgAll * msk2 (:344), while the Wiener
    // average uses fft2(imgAll) (:355-359): its sums come from the unmasked spectra, then the
    // masked copy (in xbuf; in place when imgAll lives there) replaces them for the rest.
    const float2* twid = at<float2>(ws, L.twid);
    auto spectrum = [&](const float* images) -> int {
        if (P.smem_fft) return kern::spectrum_fft(P, P.n_images, images, twid, spec, s);
        return exec_fft(P, CUFFT_R2C, P.n_images, NN, specN, const_cast<float*>(images), spec,
                        work, s);
    };
    if (!fused) MEM_STEP(spectrum(img_all));
    MEM_STEP(mark(4));
    MEM_STEP(kern::qfix(P, *in, qf, s));
    float* partial = at<float>(ws, L.partial);
    float* means = at<float>(ws, L.means);
    float2* avg_spec = at<float2>(ws, L.avg_spec);
    uint32_t* pd_max = at<uint32_t>(ws, L.pd_max);
    const SumItem* items = at<SumItem>(ws, L.sum_items);
    const int32_t* item_off = at<int32_t>(ws, L.item_off);
    const FeatTables ft = feat_tables(P, at<char>(ws, L.colmap));
    if (in->pd_mask) {
        // the Wiener average from the unmasked spectra, then everything else (centring vectors
        // included, so that they centre the features D is computed from) from the masked ones
        MEM_STEP(kern::pd_sums(P, spec, qf, items, partial, 1, s));
        MEM_STEP(kern::pd_finalize(P, partial, items, item_off, pds, ft.ring_of, means,
                                   avg_spec, pd_max, 1, s));
        MEM_STEP(kern::apply_pd_mask(P, img_all, xbuf, in->pd_mask, img_pd, s));
        MEM_STEP(spectrum(xbuf));
        MEM_STEP(kern::pd_sums(P, spec, qf, items, partial, 3, s));
        MEM_STEP(kern::pd_finalize(P, partial, items, item_off, pds, ft.ring_of, means,
                                   avg_spec, pd_max, 2, s));
    } else {
        MEM_STEP(kern::pd_sums(P, spec, qf, items, partial, 3, s));
        MEM_STEP(kern::pd_finalize(P, partial, items, item_off, pds, ft.ring_of, means,
                                   avg_spec, pd_max, 3, s));
    }
    MEM_STEP(mark(5));
    // features of D, a_i, sign(C) F, CTF output
    void* feat_a = at<char>(ws, L.feat_a);
    void* feat_b = at<char>(ws, L.feat_b);
    double* pair_norm = out->pair_norm ? out->pair_norm : at<double>(ws, L.pair_norm);
    const uint32_t* scale_bits = pd_max;
    MEM_STEP(kern::features(P, spec, qf, pds, img_pd, img_row, ft, means,
                            scale_bits, feat_a, feat_b, pair_norm, out->ctf, out->spectrum,
                            !P.smem_fft && (out->img_all_flip || out->img_all_intensity), s));
    MEM_STEP(mark(6));
    // averages: one inverse transform per PD (linearity of the reference's per-image sums)
    float* avg_real = at<float>(ws, L.avg_real);
    if (out->img_avg || out->img_avg_flip) {
        if (P.smem_fft)
            MEM_STEP(kern::inverse_fft(P, 2 * P.n_pd, avg_spec, twid, avg_real, nullptr, false, s));
        else
            MEM_STEP(exec_fft(P, CUFFT_C2R, 2 * P.n_pd, specN, NN, avg_spec, avg_real, work, s));
        MEM_STEP(kern::avg_store(P, avg_real, out->img_avg, out->img_avg_flip, in->pd_mask, s));
    }
    MEM_STEP(mark(7));
    // phase-flipped images and their mean intensity
    if (out->img_all_flip || out->img_all_intensity) {
        float* flip_imgs = out->img_all_flip ? out->img_all_flip : xbuf;
        if (P.smem_fft)
            MEM_STEP(kern::inverse_fft(P, P.n_images, spec, twid, flip_imgs, qf, true, s));
        else
            MEM_STEP(exec_fft(P, CUFFT_C2R, P.n_images, specN, NN, spec, flip_imgs, work, s));
        MEM_STEP(kern::intensity(P, flip_imgs, pds, out->img_all_intensity, s));
    }
    MEM_STEP(mark(8));
    // (a10) D
    if (!P.params.avg_only && out->D) {
        const Tile* tiles = at<Tile>(ws, L.tiles);
        if (P.params.precision == MEM_PREC_FP32)
            MEM_STEP(kern::gemm_fp32(P, (const float*)feat_a, pair_norm, scale_bits, tiles, pds,
                                     ft.chunks, out->D, s));
        else
            MEM_STEP(kern::gemm_split_bf16(P, feat_a, feat_b, pair_norm, scale_bits,
                                           at<Tile>(ws, L.tc_tiles), pds, ft.chunks, out->D,
                                           status, s));
    }
    MEM_STEP(mark(9));
#undef MEM_STEP
    return MEM_OK;
}

}  // namespace

int mem_plan_set_timing(mem_plan* plan, int enable) {
    if (!plan) return MEM_ERR_INVALID;
    if (enable && !plan->ev[0]) {
        for (auto& e : plan->ev) MEM_CUDA_TRY(cudaEventCreate(&e));
    }
    plan->timing = enable != 0;
    return MEM_OK;
}

int mem_plan_phase_times(mem_plan* plan, float* ms_out, int max_phases) {
    if (!plan || !ms_out || max_phases < 0) return MEM_ERR_INVALID;
    if (!plan->timed_run) return MEM_ERR_INVALID;
    MEM_CUDA_TRY(cudaEventSynchronize(plan->ev[MEM_NUM_PHASES]));
    const int n = std::min(max_phases, MEM_NUM_PHASES);
    for (int i = 0; i < n; ++i) {
        float ms = 0.f;
        if (plan->phase_ran[i]) MEM_CUDA_TRY(cudaEventElapsedTime(&ms, plan->ev[i], plan->ev[i + 1]));
        ms_out[i] = ms;
    }
    return MEM_NUM_PHASES;
}

const char* mem_phase_name(int phase) {
    static const char* names[MEM_NUM_PHASES] = {"gather", "lowpass", "rotate", "spectrum",
                                                "sums", "features", "averages", "flip",
                                                "contraction"};
    return (phase >= 0 && phase < MEM_NUM_PHASES) ? names[phase] : "";
}

int mem_workspace_status(const mem_plan* plan, const void* workspace) {
    if (!plan || !workspace) return MEM_ERR_INVALID;
    uint32_t st = 0;
    MEM_CUDA_TRY(cudaMemcpy(&st, static_cast<const char*>(workspace) + plan->lay.status,
                            sizeof(st), cudaMemcpyDeviceToHost));
    if (st & kStatusTimeout) return MEM_ERR_DEVICE_TIMEOUT;
    if (st & kStatusBadIndex) return MEM_ERR_INVALID;
    return MEM_OK;
}

int mem_plan_set_wait_limit(mem_plan* plan, int64_t cycles) {
    if (!plan || cycles < 1000) return MEM_ERR_INVALID;
    plan->wait_cycles = (long long)cycles;
    return MEM_OK;
}

int mem_pd_batch(const mem_params* params, int32_t n_pd, const int32_t* pd_count,
                 const double* psi_p_deg, const mem_inputs* in, const mem_outputs* out,
                 void* workspace, size_t workspace_bytes, void* stream) {
    mem_plan* plan = nullptr;
    int st = mem_plan_create(params, n_pd, pd_count, psi_p_deg, &plan);
    if (st != MEM_OK) return st;
    st = mem_plan_upload(plan, workspace, workspace_bytes, stream);
    if (st == MEM_OK) st = mem_plan_execute(plan, in, out, workspace, workspace_bytes, stream);
    mem_plan_destroy(plan);
    return st;
}

}  // extern "C"
