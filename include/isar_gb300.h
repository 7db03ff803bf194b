/*
 * isar_gb300.h -- plain C ABI of the GB300 ISAR imaging library
 * (libisar_gb300.so).  Pointers and sizes only; no C++ or torch types.
 *
 * The library re-implements the single-image imaging chain of
 * Junf137/isar_imaging_cuda (isarMainSingle -> ISAR_RD_Imaging_Main_Ku,
 * isar_imaging/isar_main.cu:3-227) on hand-written sm_103a kernels.
 * The reference's own seven exports (isar_imaging_export.h) are provided on
 * top of this ABI, see isar_imaging_export.h in this directory.
 *
 * Data layout (as the reference): complex64 interleaved (re, im) float
 * pairs, row-major [echo_num][range_num], row = pulse.  Images are float
 * [echo_num][512], row = Doppler bin, column = range bin.
 *
 * Errors: every int-returning call returns ISAR_OK (0) or a negative
 * ISAR_E* code; isar_get_last_error() gives the message of the calling
 * thread's last failure.
 */
#ifndef ISAR_GB300_H_
#define ISAR_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define ISAR_API __attribute__((visibility("default")))
#else
#define ISAR_API
#endif

enum {
    ISAR_OK = 0,
    ISAR_EINVAL = -1,   /* invalid argument or unsupported size            */
    ISAR_ECUDA = -2,    /* CUDA runtime error                              */
    ISAR_ENOMEM = -3,   /* device or host allocation failed                */
    ISAR_ESTATE = -4,   /* call out of order (e.g. no frame imaged yet)    */
    ISAR_EIO = -5       /* file I/O error (.wbd ingest)                    */
};

/* DATA_TYPE (isar_imaging/common.cuh:82-87) */
enum { ISAR_DATA_IFDS = 1, ISAR_DATA_STRETCH = 2 };

/* flags for one frame: if_hpc (isar_main.cu:33), if_mtrc (isar_main.cu:160),
 * if_hrrp (isar_main.cu:59).  The reference never returns the HRRP itself,
 * but on STRETCH data getHRRP multiplies the echoes in place by the range
 * Hamming window before range alignment (common.cu:565); ISAR_FLAG_HRRP
 * applies that window, so the image matches the reference's with if_hrrp. */
enum { ISAR_FLAG_HPC = 1, ISAR_FLAG_MTRC = 2, ISAR_FLAG_HRRP = 4, ISAR_FLAG_IQ16 = 8 };
/* ISAR_FLAG_IQ16: d_echo holds the sensor's int16 I/Q samples (2*M*N int16,
 * I and Q interleaved, as in the .wbd payload) instead of 2*M*N floats;
 * range alignment reads them directly (the reference casts them to float on
 * the host, common.cu:1096-1098).  Device-buffer entry points only. */

/* RadarParameters (isar_imaging/common.cuh:96-117) */
typedef struct {
    int echo_num;          /* M: pulses per image, power of two, 128..1024     */
    int range_num;         /* N: range cells, power of two, 512..8192, >= M    */
    long long band_width;  /* Hz                                               */
    long long fc;          /* Hz                                               */
    double Tp;             /* s                                                */
    long long Fs;          /* Hz                                               */
    int data_type;         /* ISAR_DATA_STRETCH or ISAR_DATA_IFDS              */
} isar_radar;

/* Decisions of the last imaged frame, for inspection and parity checks. */
typedef struct {
    float* ra_shift;          /* in: caller buffer of M-1 floats, or NULL    */
    float* phase;             /* in: caller buffer of 2*M floats, or NULL    */
    int center_applied;       /* HRRPCenter shifted the profiles             */
    int center_shift;         /* shift_num, cells                            */
    int cut_offset;           /* first range cell of the 512-cell cut        */
    int center_idx1_len;
    int center_idx2_len;
    float center_threshold;
    int tgt_num;              /* fastEntropy target range bins               */
    int unit2_num;            /* U, bins used by the autofocus               */
    int bins[512];            /* the U bins, ascending                       */
    int af_iterations;        /* autofocus phase updates applied (with a warm
                                 start: both legs)                           */
    float af_entropy;         /* entropy of the U bins at the last evaluated
                                 phase, with a warm start of the kept final
                                 phase (cluster engine; NaN otherwise)       */
    int ws_used;              /* the learned leg's result was kept           */
    float af_entropy_final[2];/* final entropy of the U bins of the plain leg
                                 (Doppler-tracking start) and of the learned
                                 leg (NaN without a warm start)              */
    int af_iterations_leg[2]; /* phase updates of the plain and the learned
                                 leg (0 without a warm start)                */
} isar_trace;

/*
 * Launch parameters of one context (no counterpart in the reference, whose
 * parameters are compile-time constants).  Defaults reproduce the reference:
 * 120 autofocus iterations, no stop criterion; the default autofocus engine
 * is the fastest measured for one frame of M pulses (clusters of 4, 8, 16
 * CTAs at 128, 256, 1024 pulses, the cooperative grid at 512).
 */
typedef struct {
    int ra_pair_min;          /* fused pair kernel while pairs >= this (128)          */
    int ra_rows_per_cta;      /* rows per CTA of the envelope accumulation (4)        */
    int ra_rows_final;        /* rows per CTA of the final range transform (4)        */
    int af_cluster;           /* autofocus engine: 0 = one cooperative grid of 128    */
                              /* CTAs; 4, 8, 16 = one thread-block cluster per frame  */
    float af_tol;             /* stop once the entropy of the selected bins changes   */
                              /* by <= af_tol * |entropy| per iteration (mean over 4, */
                              /* checked every 4th iteration; cluster engine; 0 = off)*/
    int af_iters;             /* autofocus iterations, or the cap with af_tol (120)   */
    int af_cluster_max;       /* out: largest af_cluster this device can launch       */
    int ra_rows_each_level;   /* range-alignment envelopes: 0 = spectral merge (one   */
                              /* spectrum per group, shifted by a phase ramp); 1 =    */
                              /* transform the shifted rows again at every level (0)  */
} isar_tuning;

typedef struct isar_ctx isar_ctx;
typedef struct isar_wsnet isar_wsnet;   /* learned warm-start network, see below */

/* Copies the calling thread's last error message; returns its length. */
ISAR_API int isar_get_last_error(char* buf, size_t len);

/* Library version string. */
ISAR_API const char* isar_version(void);

/* Number of CUDA kernels this library has launched so far (all contexts). */
ISAR_API long long isar_launch_count(void);

/*
 * Creates an imaging context on `device` for frames of radar->echo_num x
 * radar->range_num: device workspace, twiddle/window/CZT tables and a
 * stream (`stream` = an existing cudaStream_t to use, or NULL for a new one).
 * Replaces imagingMemInit (isar_imaging_export.cpp:121-205).
 */
ISAR_API int isar_create(isar_ctx** out, const isar_radar* radar, int device, void* stream);
ISAR_API int isar_destroy(isar_ctx* ctx);

/* The stream the context launches on (cudaStream_t). */
ISAR_API void* isar_stream(isar_ctx* ctx);

ISAR_API int isar_get_tuning(isar_ctx* ctx, isar_tuning* out);
/* Validates and applies `t` (af_cluster_max is ignored); drops cached graphs. */
ISAR_API int isar_set_tuning(isar_ctx* ctx, const isar_tuning* t);

/*
 * One frame from host memory: echo = 2*M*N floats, velocity = M doubles
 * (read only with ISAR_FLAG_HPC on STRETCH data, may be NULL otherwise),
 * img = M*512 floats.  Blocking, like isarMainSingle
 * (isar_imaging_export.cpp:208-212).
 */
ISAR_API int isar_image_host(isar_ctx* ctx, const float* echo, const double* velocity, int flags, float* img);

/*
 * One frame on device memory, stream-ordered on isar_stream(ctx), no host
 * synchronisation.  d_echo (2*M*N floats) is only read; the range profiles
 * (the reference's d_data_proc after range alignment) stay in the context,
 * see isar_get_profiles.  d_velocity: M doubles on the device (or NULL
 * without HPC).  d_img: M*512 floats.  d_echo must be 16-byte aligned (its
 * rows are staged into shared memory by bulk copies; cudaMalloc and torch
 * allocations are); otherwise ISAR_EINVAL.
 */
ISAR_API int isar_image_device(isar_ctx* ctx, const float* d_echo, const double* d_velocity, int flags, float* d_img);

/* Waits for the context stream and reports a device-side failure of the
 * frames queued so far (e.g. a timed-out grid barrier) as ISAR_ECUDA. */
ISAR_API int isar_synchronize(isar_ctx* ctx);

/* Device pointer of the context's M*N complex range profiles of the last
 * frame (aligned, before centering). */
ISAR_API int isar_get_profiles(isar_ctx* ctx, const float** d_profiles);

/* Decisions of the last frame (synchronises the context stream). */
ISAR_API int isar_get_trace(isar_ctx* ctx, isar_trace* out);

/* ---- stage entry points (device pointers, stream-ordered, in place) ---- */

/* highSpeedCompensation (high_speed_compensation.cu:4-54) applied to d_x. */
ISAR_API int isar_stage_hpc(isar_ctx* ctx, float* d_x, const double* d_velocity);
/* rangeAlignmentParallel (range_alignment.cu:4-78), with HPC fused in when
 * flags has ISAR_FLAG_HPC: spectra in d_x -> complex range profiles.
 * d_x must be 16-byte aligned. */
ISAR_API int isar_stage_range_align(isar_ctx* ctx, float* d_x, const double* d_velocity, int flags);
/* HRRPCenter (range_alignment.cu:371-465) + cutRangeProfile
 * (common.cu:494-509): profiles d_y (M*N) -> d_cut (M*512). */
ISAR_API int isar_stage_center_cut(isar_ctx* ctx, const float* d_y, float* d_cut);
/* getHRRP (common.cu:541-580): the M*N complex high-resolution range
 * profiles of the echoes d_x into d_hrrp (may equal d_x): STRETCH rows are
 * FFT(x * hamming) with the halves swapped, IFDS rows swap, FFT, swap.  The
 * reference computes them when if_hrrp is set and keeps them on the device;
 * here they are a stage of their own (the windowing that if_hrrp applies to
 * the STRETCH echoes is ISAR_FLAG_HRRP). */
ISAR_API int isar_stage_hrrp(isar_ctx* ctx, const float* d_x, float* d_hrrp);
/* fastEntropy (phase_adjustment.cu:167-332) in place on d_cut. */
ISAR_API int isar_stage_fast_entropy(isar_ctx* ctx, float* d_cut, int iterations);
/* mtrc (mtrc.cu:4-76, when ISAR_FLAG_MTRC) and post-processing
 * (isar_main.cu:191-211): d_cut -> d_img (M*512 floats). */
ISAR_API int isar_stage_post(isar_ctx* ctx, float* d_cut, int flags, float* d_img);

/* ---- synthetic dechirped echoes (benchmarks, training data) ------------ */
typedef struct {
    int M, N;                 /* pulses, range cells                              */
    double fc, B, prf, Fs;    /* Hz                                               */
    int n_scat;               /* point scatterers (Rayleigh amplitudes)           */
    double patch_x, patch_y;  /* m: cross-range, range extent of the target patch */
    double omega;             /* rad/s rotation rate                              */
    double r0_cells;          /* range offset of the patch centre, cells          */
    double drift_sigma;       /* cells: per-pulse random-walk range drift         */
    double phase_uniform;     /* rad: half width of the uniform phase error       */
    double phase_quad;        /* rad: quadratic phase error at the aperture edge  */
    double v0, accel;         /* m/s, m/s^2: radial velocity (HPC term)           */
    double snr_db;
    double rms_counts;        /* ADC scale of the signal part (int16 counts)      */
    uint64_t seed;
    int phase_poly_order;     /* >= 2: add sum_{k=2..order} c_k u^k, u in [-1,1) */
    double phase_poly_sigma;  /* rad: c_k ~ N(0, sigma), drawn per frame          */
    double* h_phase_err;      /* out (host, M doubles, may be NULL): per-pulse    */
                              /* phase to remove, rad: the injected error plus    */
                              /* the carrier phase of the range drift             */
} isar_synth_params;

/* Writes one M x N frame of int16-quantised counts as complex64 into d_out
 * (device), the quantised per-pulse velocities into d_velocity (device,
 * may be NULL) and h_velocity (host, may be NULL).  Blocking on `stream`. */
ISAR_API int isar_synth_device(const isar_synth_params* p, float* d_out, double* d_velocity, double* h_velocity,
                               void* stream);

/* Test hook: make range alignment use the given M-1 shifts (level-major, as
 * isar_trace.ra_shift) instead of its own estimates; NULL restores normal
 * operation.  Isolates the rest of the chain from the float rounding of the
 * reference's parabolic shift estimate in parity tests. */
ISAR_API int isar_set_ra_shifts(isar_ctx* ctx, const float* shifts);

/* Test hook for the bounded device waits that replace the reference's
 * exit() on a CUDA error (helper_cuda.h:583-595): the cooperative autofocus
 * engine's grid barrier gives up after `polls` polls (0 = the default limit,
 * about a second) and, with never_complete != 0, waits for one arrival more
 * than the grid makes, so that every CTA gives up, sets the timeout flag and
 * leaves the kernel.  The frame then reports ISAR_ECUDA and the context stays
 * usable.  (0, 0) restores normal operation. */
ISAR_API int isar_test_barrier_timeout(isar_ctx* ctx, unsigned polls, int never_complete);

/*
 * HRRPCenter + cutRangeProfile without a context and without allocating:
 * the same computation as isar_stage_center_cut, profiles d_profiles
 * (echo_num x range_num complex, device) -> d_cut (echo_num x 512 complex,
 * device), stream-ordered on `stream` (NULL = the legacy default stream),
 * which must belong to the calling thread's current device.  No counterpart
 * in the reference: it is for callers that cannot allocate device memory
 * (a fixed, pre-reserved memory budget; cudaMalloc/cudaFree, which can
 * synchronise the device, are not allowed inside their processing loop).
 *
 * Sizes are those of isar_create: echo_num a power of two in [128, 1024],
 * range_num a power of two in [512, 8192].  Scratch is one static device
 * array per device, sized for range_num <= 8192; larger range_num returns
 * ISAR_EINVAL.  The first call on
 * each device sets up (symbol address and a kernel attribute, no allocation);
 * make that first call before capturing a stream, e.g. with all arguments
 * NULL/0, which performs the set-up only.  Calls that overlap in time on one
 * device (different streams or threads) share the scratch and race: order
 * them, e.g. on one stream.
 */
ISAR_API int isar_center_cut_noalloc(const float* d_profiles, int echo_num, int range_num, float* d_cut,
                                     void* stream);

/*
 * Autotuner (no counterpart in the reference): times whole frames of
 * d_echo on this context over the range-alignment knobs (envelope path, then
 * the carried-envelope path's pair threshold and rows per CTA when that path
 * wins, then the final transform's rows per CTA) and the autofocus
 * engines allowed by `engines` (bit 0: cooperative grid, bit 1: clusters),
 * coordinate by coordinate, applies the fastest and returns it.  Keeps
 * af_tol and af_iters.  Blocking; allocates a scratch image while it runs.
 */
ISAR_API int isar_autotune(isar_ctx* ctx, const float* d_echo, const double* d_velocity, int flags, int engines,
                           isar_tuning* out);

/* ---- batches: many frames of uneven size in one CUDA graph ---------------
 * No counterpart in the reference (one frame per isarMainSingle).  Frames are
 * grouped by isar_radar; each group is dealt round-robin to `lanes` contexts
 * with their own streams; the whole batch is captured once into a CUDA graph
 * (fork/join on the batch stream) and replayed.  Lanes use the cluster
 * autofocus engine.  Results equal those of isar_image_device with the same
 * isar_tuning. */
typedef struct {
    isar_radar radar;         /* M, N and radar parameters of this frame         */
    const float* d_echo;      /* device, 2*M*N floats, read only, 16-byte aligned */
    const double* d_velocity; /* device, M doubles (ISAR_FLAG_HPC), or NULL      */
    int flags;                /* ISAR_FLAG_*                                     */
    float* d_img;             /* device, M*512 floats                            */
} isar_batch_frame;

typedef struct isar_batch isar_batch;

/* lanes: contexts per frame shape, 0..128 (0 = 4); `stream` = cudaStream_t or NULL. */
ISAR_API int isar_batch_create(isar_batch** out, int device, void* stream, int lanes);
ISAR_API int isar_batch_destroy(isar_batch* b);
ISAR_API void* isar_batch_stream(isar_batch* b);
/* Stream-ordered on isar_batch_stream(b); the graph is cached per frame list. */
ISAR_API int isar_batch_run(isar_batch* b, const isar_batch_frame* frames, int n);
/* Waits for the batch and reports device-side failures. */
ISAR_API int isar_batch_synchronize(isar_batch* b);
ISAR_API int isar_batch_set_tuning(isar_batch* b, const isar_radar* shape, const isar_tuning* t);
ISAR_API int isar_batch_get_tuning(isar_batch* b, const isar_radar* shape, isar_tuning* out);
ISAR_API int isar_batch_lanes(isar_batch* b);
/* Attaches `net` (NULL detaches) as the warm start of every lane, present
 * and future (isar_set_warmstart); drops cached graphs. */
ISAR_API int isar_batch_set_warmstart(isar_batch* b, const isar_wsnet* net);
/* Tunes each shape (isar_autotune, cluster engine), then on the whole frame
 * list the lanes per shape (powers of two up to 128) with the autofocus
 * cluster size (16, 8 or 4 CTAs), then the range-alignment envelope path and
 * rows per CTA, by timing whole-batch graph replays; *best_ms (may be NULL)
 * = the fastest batch time. */
ISAR_API int isar_batch_autotune(isar_batch* b, const isar_batch_frame* frames, int n, float* best_ms);

/* ---- learned autofocus warm start ----------------------------------------
 * No counterpart in the reference.  A small network (6 x 1-D conv k=5, 64
 * channels, then a per-pulse 64 -> 64 -> 2 head) reads per-pulse features of
 * the cut (unit phasors and magnitudes of pulse-pair products on the 16
 * strongest bins, the Doppler-tracking increment psi) and predicts the
 * residual r of the Doppler-tracking phase increment.  The warm start
 * phase[m+1] = exp(-j sum (psi - r)) competes with the Doppler start: the
 * cluster engine keeps the one with the lower entropy of the selected bins.
 * Dense layers are bf16 tcgen05 GEMMs with fp32 accumulation, for inference
 * and training. */

/* Number of fp32 parameters (canonical order: 6 conv layers W[64][320] with
 * column k*64+c then b[64]; head W[64][64], b[64]; W[2][64], b[2]). */
ISAR_API int isar_wsnet_param_count(void);
/* max_rows = frames * pulses per call (multiple of 8); training != 0 keeps
 * activations and gradient buffers.  Parameters start at zero. */
ISAR_API int isar_wsnet_create(isar_wsnet** out, int max_rows, int training, int device, void* stream);
ISAR_API int isar_wsnet_destroy(isar_wsnet* net);
ISAR_API void* isar_wsnet_stream(isar_wsnet* net);
ISAR_API int isar_wsnet_set_params(isar_wsnet* net, const float* h_params);
ISAR_API int isar_wsnet_get_params(isar_wsnet* net, float* h_params);
/* d_x0: bf16 [frames*M][64] features (isar_frame_features); d_out: fp32
 * [frames*M][2] = (c, s), r = atan2(s, c); may be NULL.  Blocking. */
ISAR_API int isar_wsnet_forward(isar_wsnet* net, const void* d_x0, int frames, int M, float* d_out);
/* Loss 1 - |mean_m exp(j (r_hat_m - r_m))| per frame (m < M-1) of the last
 * forward against d_target (fp32 [frames*M]); gradients into the network;
 * *h_loss = mean over frames (may be NULL).  Blocking. */
ISAR_API int isar_wsnet_backward(isar_wsnet* net, const float* d_target, int frames, int M, float* h_loss);
ISAR_API int isar_wsnet_get_grads(isar_wsnet* net, float* h_grads);
ISAR_API int isar_wsnet_adam(isar_wsnet* net, float lr);
/* Test entry: C[M][N] = A[M][K] * B[N][K]^T, bf16 in, fp32 out, tensor cores. */
ISAR_API int isar_nn_gemm_bf16(const void* A, int lda, const void* B, int ldb, float* C, int ldc, int M, int N, int K,
                               int splits, void* stream);

/* Attaches `net` (NULL detaches) as this context's warm start; needs the
 * cluster autofocus engine.  The network must outlive the attachment and
 * must not be trained while frames that use it are in flight. */
ISAR_API int isar_set_warmstart(isar_ctx* ctx, const isar_wsnet* net);
/* Training data: range alignment, centring, cut and the bin selection of a
 * frame, then its features d_x0 (bf16 [M][64]) and psi (fp32 [M]).
 * Stream-ordered on the context stream. */
ISAR_API int isar_frame_features(isar_ctx* ctx, const float* d_echo, const double* d_velocity, int flags, void* d_x0,
                                 float* d_psi);

/* Batched unnormalised row FFTs of length n (512..8192) in place, for tests. */
ISAR_API int isar_fft_rows(isar_ctx* ctx, float* d_x, int rows, int n, int inverse);

/* ---- sensor samples ---------------------------------------------------------
 * int16 I/Q pairs (the .wbd payload, I and Q interleaved) to complex64, on
 * the device: d_iq = 2*samples int16 (8-byte aligned), d_echo = 2*samples
 * floats (16-byte aligned), stream-ordered on `stream` (cudaStream_t or NULL).
 * The conversion the reference's getSignalData does on the host
 * (common.cu:1096-1098), so that a caller can move 4 bytes per sample. */
ISAR_API int isar_iq16_to_c64(const int16_t* d_iq, float* d_echo, size_t samples, void* stream);

/* ---- IFDS ingest ----------------------------------------------------------
 * Matched-filter pulse compression of `pulses` IFDS pulses, the
 * reference's pulseCompression::pulseCompressionbyFFT (common.cu:635-746) as
 * multiThreadIFDS drives it (common.cu:583-604), in one launch (one CTA per
 * pulse).  d_ad: pulses x 2*iq_len int16 samples, I and Q interleaved
 * (4-byte aligned); d_velocity: pulses doubles, m/s (the reference's
 * per-pulse dataNOut entry); d_out: pulses x 4096 complex (2*4096 floats per
 * pulse, RANGE_NUM_IFDS_PC), the 4096 cells around the maximum of each
 * compressed pulse (cutRangeProfile, common.cu:494-509); d_offsets (may be
 * NULL): the first cell of each cut.  B, fc, Tp and Fs come from the
 * context's radar.  NFFT = nextPow2(iq_len) (twice iq_len for a power of
 * two) must be 4096, 8192 or 16384, and (int)(Fs * Tp) in [2, NFFT].
 * Stream-ordered on isar_stream(ctx). */
ISAR_API int isar_pulse_compress(isar_ctx* ctx, const int16_t* d_ad, int iq_len, const double* d_velocity,
                                 int pulses, float* d_out, int* d_offsets);

#ifdef __cplusplus
}
#endif

#endif /* ISAR_GB300_H_ */
