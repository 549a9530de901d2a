/*
 * manifoldem_gb300.h -- C ABI of the GB300 (sm_103a) per-projection-direction distance stage.
 *
 * One call processes a batch of projection directions (PDs).  For every PD it does what
 * ManifoldEM's getDistanceCTF_local_Conj9combinedS2.op() does to the PD's particle images
 * (reference modules/getDistanceCTF_local_Conj9combinedS2.py:216-420):
 *   read each image from a SPIDER raw float32 stack (transposed, conjugate views flipped
 *   up-down), normalise it by the mean/std of its background, Butterworth-filter it, mask it,
 *   rotate it twice (periodic cubic B-spline, angles -deg(Psi_i) then -psi_p), build its CTF,
 *   and produce:
 *     D[i][j] = sum_k |CTF_j(k) F_i(k) - CTF_i(k) F_j(k)|^2      (float64, n x n per PD)
 *     imgAvg   (Wiener average), imgAvgFlip (phase-flipped average), imgAllIntensity
 *     imgAll, imgAllFlip, CTF per image (float32; the reference stores them as float64).
 *
 * Conventions
 *   - All array arguments are device pointers unless marked HOST.
 *   - The caller allocates every device buffer, including the workspace; the library keeps only
 *     host-side state (plans, cached cuFFT plans).  Nothing here calls cudaMalloc.
 *   - Every function returns MEM_OK (0) or a negative MEM_ERR_* status; nothing throws.
 *   - Work is enqueued on the caller's stream (a cudaStream_t passed as void*); mem_plan_execute
 *     issues only kernel launches and cuFFT executions, so it may be captured in a CUDA graph.
 *   - Host-side geometry (PD, PDs, Psi_i, Nom, Dnom, psi_p, imgLabels) stays with the caller, as in
 *     the reference, which computes it in numpy/scipy (:297-323, psi_ang :206-213 via
 *     q2Spider.op's least-squares fit).  The caller passes Psi_i and psi_p in.
 */
#ifndef MANIFOLDEM_GB300_H
#define MANIFOLDEM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MEM_ABI_VERSION 5

/* status codes */
#define MEM_OK                    0
#define MEM_ERR_INVALID          -1  /* bad argument (null pointer, size out of range)          */
#define MEM_ERR_UNSUPPORTED      -2  /* box size or option this library does not support         */
#define MEM_ERR_WORKSPACE        -3  /* workspace smaller than mem_plan_workspace_size()        */
#define MEM_ERR_CUDA             -4  /* a CUDA runtime call failed                               */
#define MEM_ERR_CUFFT            -5  /* a cuFFT call failed                                      */
#define MEM_ERR_DEVICE_TIMEOUT   -6  /* a bounded device-side wait expired (kernel returned)     */
#define MEM_ERR_NO_DEVICE        -7  /* no sm_103 device is current                              */
#define MEM_ERR_TOO_LARGE        -8  /* problem larger than the static scratch of the no-allocation
                                        entry point (MEM_NOALLOC_SCRATCH_BYTES)                    */

/* contraction forms for D */
#define MEM_PREC_FP32        0   /* plain FP32 SIMT contraction, FP64 epilogue                   */
#define MEM_PREC_SPLIT_BF16  1   /* 3-term split-BF16 on tcgen05 tensor cores, FP64 epilogue     */

/* low-pass filter types, filterPar['type'] (reference :156-167) */
#define MEM_FILTER_BUTTER 0
#define MEM_FILTER_GAUSS  1

/* Microscope and stage parameters: the reference's module globals p.nPix, p.pix_size, p.Cs,
 * p.EkV, p.gaussEnv, p.AmpContrast, plus filterPar and options['avgOnly'].               */
typedef struct mem_params {
    int32_t N;              /* box size (p.nPix), 8 <= N <= 512 (above 236 px the rotation
                               keeps its spline coefficients in global memory)                */
    int32_t filter_type;    /* MEM_FILTER_*                                                  */
    double  filter_Qc;      /* cutoff in units of Nyquist (filterPar['Qc'])                   */
    double  filter_order;   /* Butterworth order (filterPar['N'])                             */
    double  pix_size;       /* Angstrom per pixel                                              */
    double  Cs;             /* spherical aberration, mm                                        */
    double  EkV;            /* acceleration voltage, kV                                        */
    double  gaussEnv;       /* Gaussian envelope half-width, 1/A; +inf disables the envelope   */
    double  AmpContrast;    /* amplitude contrast ratio                                        */
    int32_t avg_only;       /* options['avgOnly']: skip D                                      */
    int32_t precision;      /* MEM_PREC_*                                                      */
} mem_params;

/* Per-call device inputs.  Images of PD p are the pd_count[p] consecutive entries starting at
 * the sum of the previous counts, in the order of the PD's index list ``ind``.           */
typedef struct mem_inputs {
    const float*   stack;        /* SPIDER raw stack, num_stack * N * N float32: device memory,
                                    or host memory the GPU can read (pinned / registered, or
                                    any host memory on a system whose GPU uses the host page
                                    tables); only the first kernel reads it, once per image   */
    int64_t        num_stack;
    const int64_t* stack_index;  /* [n_images] stack image of each entry: ind, or
                                    ind - nStot/2 for conjugate views (reference :247-252)      */
    const uint8_t* flip;         /* [n_images] 1 for conjugate views (ind >= nStot/2)         */
    const double*  psi_rad;      /* [n_images] Psi_i = 2 atan(s/c), NaN replaced by 0 (:317-321) */
    const double*  df;           /* [n_images] defocus, Angstrom                               */
    const double*  shift_yx;     /* NULL: SPIDER stack (image idx is the stored N x N block,
                                    transposed, :254-257).  Else RELION stack (:259-264): the
                                    stored image as is, shifted by [n_images][2] =
                                    (sh_y - 0.5, sh_x - 0.5) of its particle with the order-3
                                    'wrap' spline shift of scipy.ndimage; N <= 236            */
    const uint8_t* pd_mask;      /* NULL, or [n_pd][N][N] projected volume mask msk2 of every PD
                                    (mem_mask_project; reference :303-310): multiplies each
                                    rotated image before its spectrum (:344)                  */
} mem_inputs;

/* Per-call device outputs; any pointer may be NULL to skip that output.                   */
typedef struct mem_outputs {
    double* D;                 /* PD p at offset sum_{q<p} n_q^2, row-major n_p x n_p         */
    double* img_avg;           /* [n_pd][N][N]  imgAvg                                         */
    double* img_avg_flip;      /* [n_pd][N][N]  imgAvgFlip                                     */
    double* img_all_intensity; /* [n_pd][N][N]  imgAllIntensity                                */
    float*  img_all;           /* [n_images][N][N] imgAll                                      */
    float*  img_all_flip;      /* [n_images][N][N] imgAllFlip                                  */
    float*  ctf;               /* [n_images][N][N] CTF, full plane, FFT (ifftshifted) order    */
    float*  spectrum;          /* [n_images][N][N/2+1] complex (re,im) half-plane fft2(imgAll)  */
    double* pair_norm;         /* [n_images] per-image FP64 term a_i of D_ij = a_i + a_j + E_ij */
} mem_outputs;

typedef struct mem_plan mem_plan;   /* opaque */

/* ---- library ------------------------------------------------------------------------- */
int         mem_abi_version(void);
const char* mem_status_string(int status);

/* ---- plans ----------------------------------------------------------------------------
 * mem_plan_create replaces the per-PD job set-up of GetDistancesS2.op / divide()
 * (modules/GetDistancesS2.py:37-47, :94) for a batch of PDs: it fixes the box size, the PD
 * sizes and psi_p of every PD (HOST arrays), lays out the workspace and builds the tile
 * schedule of the D contraction.                                                          */
int mem_plan_create(const mem_params* params, int32_t n_pd,
                    const int32_t* pd_count /* HOST [n_pd] */,
                    const double* psi_p_deg /* HOST [n_pd], psi_ang(PD) in degrees */,
                    mem_plan** out_plan);
int mem_plan_destroy(mem_plan* plan);
int mem_plan_workspace_size(const mem_plan* plan, size_t* bytes);
int64_t mem_plan_num_images(const mem_plan* plan);
int64_t mem_plan_d_elements(const mem_plan* plan);   /* sum n_p^2 */
int64_t mem_plan_num_pairs(const mem_plan* plan);    /* sum n_p (n_p - 1) / 2 */

/* Schedule of the split-BF16 tensor-core contraction for one size class of PDs: the classes
 * are given in increasing max_n; a PD of n images belongs to the first class with
 * n <= max_n (the last class takes every larger PD).  The tiles of each class run in one
 * launch with the class's schedule.  The reference has no counterpart (its D is one float64
 * GEMM per PD, modules/getDistanceCTF_local_Conj9combinedS2.py:391-397); the schedules are
 * picked per box size and class by the autotuner (manifoldem_python_gb300/autotune.py).   */
typedef struct mem_contraction_config {
    int32_t max_n;          /* largest PD (images) of the class                                */
    int32_t persistent;     /* 0: one CTA per 128 x 128 tile; 1: one CTA per SM walking tiles   */
    int32_t accumulators;   /* TMEM accumulation buffers, 2 or 4 (the MMA issuer may run this
                               many accumulation groups ahead of the epilogue, across tiles);
                               2 with 256-wide tiles                                          */
    int32_t tile_n;         /* D columns per tile: 128, or 256 (128 x 256 tiles: a quarter
                               fewer operand bytes per MMA, two 96 KB stages instead of three
                               64 KB ones); 0 means 128                                        */
    int32_t tile_m;         /* D rows per tile: 128 (one SM), or 256 (a pair of SMs sharing
                               one MMA stream, tcgen05.mma.cta_group::2: each SM loads 128 A
                               rows and half of the 128 B rows, 48 KB per K chunk, four stages;
                               needs tile_n 128); 0 means 128                                  */
    int32_t reserved;       /* 0                                                               */
} mem_contraction_config;

/* Sets the plan's contraction schedule (HOST array of n_classes >= 1 entries, max_n
 * strictly increasing); call before mem_plan_upload.  Default: one class, one CTA per tile,
 * two accumulators, 128-wide tiles.  MEM_ERR_INVALID on a malformed table or after the
 * upload.                                                                                  */
int mem_plan_set_contraction(mem_plan* plan, int32_t n_classes,
                             const mem_contraction_config* classes);

/* Copy the plan's tables into the workspace (stream-ordered).  Call once per workspace
 * before mem_plan_execute (and before capturing it).                                      */
int mem_plan_upload(mem_plan* plan, void* workspace, size_t workspace_bytes, void* stream);

/* The distance stage for every PD of the plan: replaces
 * getDistanceCTF_local_Conj9combinedS2.op (modules/getDistanceCTF_local_Conj9combinedS2.py:216)
 * for the PDs of the plan, minus its pickle write (myio.fout1, :409-412), which stays with the
 * caller.  Stream-ordered and graph-capturable.                                            */
int mem_plan_execute(mem_plan* plan, const mem_inputs* in, const mem_outputs* out,
                     void* workspace, size_t workspace_bytes, void* stream);

/* mem_plan_execute with the reading of the stack issued on load_stream and the rest of the stage
 * on stream, which waits for it (an event owned by the plan).  With the stack in host memory
 * the load stream only copies the entries' images over the host link into free workspace
 * slots (8 CTAs of 1024 threads without shared memory, MEM_HOST_LOAD_CTAS /
 * MEM_HOST_LOAD_THREADS: few SMs, enough loads in flight for the link), so the loads of one plan
 * overlap the computation of other plans on other streams; a device-resident stack is read by
 * the first kernel of the stage on load_stream.  The reference has no counterpart (its workers
 * read the stack from disk, :255-283).  Not for graph capture.                              */
int mem_plan_execute_split(mem_plan* plan, const mem_inputs* in, const mem_outputs* out,
                           void* workspace, size_t workspace_bytes, void* load_stream,
                           void* stream);

/* Reads the device status word of the workspace (after the stream has been synchronised):
 * MEM_OK; MEM_ERR_DEVICE_TIMEOUT if a bounded device-side wait gave up (the kernel returned
 * early, its outputs are incomplete); MEM_ERR_INVALID if an entry's stack_index was outside
 * [0, num_stack) (never dereferenced; that image's outputs are NaN).  The word is cleared at
 * the start of every execute.                                                              */
int mem_workspace_status(const mem_plan* plan, const void* workspace);

/* Limit of the bounded device-side waits of the plan's kernels (the tensor-core contraction's
 * mbarrier waits), in SM clock cycles; default 4e9 (~2 s at 2 GHz), at least 1000.  A wait
 * that runs out sets the status word's timeout bit, the kernel stops issuing, waits (bounded)
 * for its own copies and MMAs in flight, frees its tensor memory and returns.  The reference
 * has no counterpart (it has no device code).  Applies to executes enqueued afterwards.     */
int mem_plan_set_wait_limit(mem_plan* plan, int64_t cycles);

/* ---- phase timing ------------------------------------------------------------------------
 * When enabled, mem_plan_execute records CUDA events between its phases (gather, lowpass,
 * rotate, spectrum, sums, features, averages, flip, contraction).  mem_plan_phase_times waits
 * for the last execute's events and writes up to max_phases durations in milliseconds (phases
 * that did not run report 0); it returns the number of phases.  Keep timing disabled while
 * capturing a graph.                                                                        */
#define MEM_NUM_PHASES 9
int mem_plan_set_timing(mem_plan* plan, int enable);
int mem_plan_phase_times(mem_plan* plan, float* ms_out, int max_phases);
const char* mem_phase_name(int phase);

/* One-shot convenience: plan, upload and execute on `stream`, then destroy the plan.
 * The workspace must be at least the size mem_plan_workspace_size reports for the same
 * arguments.                                                                               */
int mem_pd_batch(const mem_params* params, int32_t n_pd, const int32_t* pd_count,
                 const double* psi_p_deg, const mem_inputs* in, const mem_outputs* out,
                 void* workspace, size_t workspace_bytes, void* stream);

/* ---- no-allocation entry point ---------------------------------------------------------
 * No counterpart in the reference (which has no GPU path).  For callers that cannot allocate
 * device memory at all -- a plugin running inside a host application that owns every device
 * buffer and grants no allocation rights, code called back from another runtime's memory pool,
 * or a latency-critical path that must not pay for cudaMalloc or fragment the heap -- this
 * computes D for ONE PD from the PD's half-plane spectra (the mem_outputs.spectrum layout,
 * fft2(imgAll) as (re, im) float pairs, [n][N][N/2+1]) and defocus values, with every
 * intermediate in a file-scope static device array of MEM_NOALLOC_SCRATCH_BYTES.  It calls no
 * cudaMalloc, cudaFree or allocating library routine (no cuFFT).
 *   - spectra, df (device, [n]) and D (device, n*n doubles, row-major) are the caller's;
 *     params->avg_only is ignored; params->precision selects the contraction form.
 *   - The first call on a device resolves the array's device address and the SM count on that
 *     device (make it current first); make that first call before any stream capture.  The
 *     first call on a device and the first call after a change of box size also copy the box
 *     size's feature-layout tables from host memory into the array; make those calls before
 *     any stream capture too.  The other per-call tables are written by a kernel.
 *   - The resolved address assumes the device's context lives until the process exits: a
 *     cudaDeviceReset between calls is not supported.
 *   - Sizes whose scratch (feature matrix rows padded to 128, spectra copy, sums) would exceed
 *     MEM_NOALLOC_SCRATCH_BYTES return MEM_ERR_TOO_LARGE without launching anything; at 128 px
 *     that allows n <= 187 images, at 70 px n <= 692; boxes above 220 px do not fit.
 *   - Every call on a device shares the one array and it keeps the last call's contents (the
 *     call re-initialises what it needs); calls that overlap on the GPU (other streams, other
 *     host threads) race on it and must be serialised by the caller.                          */
#define MEM_NOALLOC_SCRATCH_BYTES (32u << 20)
int mem_pd_distances_noalloc(const mem_params* params, int32_t n, const float* spectra,
                             const double* df, double* D, void* stream);

/* Status of the last mem_pd_distances_noalloc call on the current device (no counterpart in
 * the reference; it allocates nothing either): waits for `stream`
 * (the stream that call was enqueued on), then reads the status word kept at the start of the
 * static scratch array (no allocation).  MEM_OK, or MEM_ERR_DEVICE_TIMEOUT when a bounded
 * device-side wait of the split-BF16 contraction gave up (D is then incomplete).           */
int mem_noalloc_status(void* stream);

/* ---- diffusion-map embedding of one PD's D (the stage's consumer) -----------------------
 * The dense-matrix work of DMembeddingII.op (modules/DMembeddingII.py:86-185) with
 * fergusonE.op (modules/fergusonE.py:33-58) and slaplacianonFly.op (:42-81), on device memory;
 * the caller keeps the neighbour lists, the tanh fit and the eigen-decomposition (as the Python
 * op in manifoldem_python_gb300/DMembeddingII.py does).
 *
 * mem_dm_symmetrise: Y (n x n f64) from D (n x n f64): the reference's symmetrised list of
 *   squared distances (DMembeddingII.py:112-139): s_ij = sqrt(D_ji) when j is a listed neighbour
 *   of point i (listed[i*n + j] != 0; listed == NULL lists every point, k = n), D_ji >= 1e-6 and
 *   j != i, else 0; Y_ij = s_ij^2 + s_ji^2 - s_ij s_ji; entries that are not edges are -1.
 * mem_dm_sweep: sums[e] = sum over edges (Y >= 0) of exp(-d), d = Y/(2 eps_e), over the terms
 *   with d < thr (fergusonE.py:36-44); scale[e] = log2(e)/(2 eps_e) (device, float32, at most
 *   2048 values).  exp in float32, sums in float64.
 * mem_dm_laplacian: Y becomes the symmetric normalised kernel L of slaplacianonFly (alpha = 1):
 *   W = exp(-Y/sigma^2) on edges, W'_ij = W_ij/(d_i d_j) (d = column sums of W),
 *   L_ij = W'_ij/(e_i e_j) (e = sqrt(column sums of W')), L = |L + L^T|/2; scratch holds 2n
 *   doubles.                                                                                */
int mem_dm_symmetrise(const double* D, int64_t n, const uint8_t* listed, double* Y,
                      void* stream);
int mem_dm_sweep(const double* Y, int64_t n, const float* scale, int32_t n_eps, double thr,
                 double* sums, void* stream);
int mem_dm_laplacian(double* Y, int64_t n, double sigma, double* scratch, void* stream);

/* ---- volume mask (reference :303-310, projectMask.op modules/projectMask.py:118-135) ------
 * mem_mask_prepare: spline coefficients of the mask volume (device, (N, N, N) float32 as
 *   stored, z y x) for projectMask's order-3 'nearest' affine_transform: axes 0 and 2 swapped,
 *   padded by 12 edge samples per side, 'reflect' prefiltered; coeffs holds
 *   mem_mask_coefficients_size bytes (float64, (N+24)^3).  N <= 236.
 * mem_mask_project: for every PD p, masks[p] (N x N bytes, 0/1) = projectMask.op of the volume:
 *   transforms[p] = R row-major (9 doubles) and offset (3) of the PD's affine map (output voxel
 *   o samples the volume at R o + offset; manifoldem_python_gb300.geometry.mask_transform);
 *   device pointers.  Float64 throughout.                                                    */
int mem_mask_coefficients_size(int32_t N, size_t* bytes);
int mem_mask_prepare(const float* volume, int32_t N, double* coeffs, void* stream);
int mem_mask_project(const double* coeffs, int32_t N, int32_t n_pd, const double* transforms,
                     uint8_t* masks, void* stream);

/* ---- NLSA snapshot stage (reference modules/NLSA.py:23-158, get_wiener.py:9-21) ------------
 * The per-PD arrays of NLSA.op that scale with the images; the caller keeps the two embeddings,
 * the small SVD and the curve fit (as manifoldem_python_gb300/NLSA.py does).  Device pointers,
 * row-major.  num = images in the PD, c = ConOrder (1 <= c < num), m = num - c.
 *
 * mem_nlsa_con_distances: ConD (m x m f64) = sum_{i < c} DD[i:i+m, i:i+m] (DD num x num f64),
 *   added in order i = 0, 1, .. from 0 (NLSA.py:31-34): bit-identical to the reference.
 * mem_nlsa_snapshots: A (c N^2 x n_modes f64) of NLSA.py:63-86, block ii (rows ii N^2 ..) =
 *   tmp_ii mu_psi with column i of tmp_ii the snapshot j = c - ii + i - 1 transposed and
 *   flattened (row x N + y holds pixel [y][x]):
 *     ctf != NULL (the 'prD' branch): snapshot = msk2 * Re ifft2(fft2(images[j]) ctf[j] / wd_i),
 *       wd_i = sum_{t = i+1 .. i+c} ctf[t]^2 + 1/5 (get_wiener.py), msk2 (N x N f64) or NULL
 *       for 1.  ctf[j] must be even in frequency, as every CTF of the distance stage is
 *       (C(-k) = C(k) on the ifftshifted grid); the Wiener sum runs over half-plane spectra.
 *     ctf == NULL (the 'cuti' branch): snapshot = images[j], no filter and no mask.
 *   images, ctf: (num, N, N) float32 as stored (ctf ifftshifted); mu_psi: m x n_modes f64.
 *   Spectra and the banded Wiener sum in float32 with float64 Wiener denominators; A float64.
 *   workspace: mem_nlsa_workspace_size bytes.  N <= 512, 1 <= n_modes <= 64.                */
int mem_nlsa_con_distances(const double* DD, int32_t num, int32_t c, double* ConD, void* stream);
int mem_nlsa_workspace_size(int32_t N, int32_t num, int32_t c, int32_t n_modes, int32_t wiener,
                            size_t* bytes);
int mem_nlsa_snapshots(int32_t N, int32_t num, int32_t c, int32_t n_modes, const float* images,
                       const float* ctf, const double* mu_psi, const double* msk2,
                       void* workspace, size_t workspace_bytes, double* A, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* MANIFOLDEM_GB300_H */
