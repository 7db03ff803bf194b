/*
 * isar_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * FP64, single-threaded CPU restatement of the Junf137/isar_imaging_cuda
 * single-image ISAR chain (isarMainSingle -> ISAR_RD_Imaging_Main_Ku):
 * high-speed compensation, range alignment, HRRP centering + cut,
 * Doppler tracking + fast minimum-entropy autofocus, CZT MTRC, post.
 *
 * This is the checker the CUDA path is compared against and the timed CPU
 * baseline.  Only tests, __graft_entry__.smoke() and bench.py's CPU legs use it;
 * the product library never links it.
 *
 * Pinning: the restatement is checked against golden vectors produced by the
 * reference's own source code (its kernels, control flow and Thrust calls)
 * executed on the CPU through a CUDA-runtime emulation shim, see
 * oracle/ref_emu/ and tests/golden/make_golden.py.
 *
 * Conventions (all as in the reference):
 *   data: complex, row-major [echo_num][range_num] (row = pulse);
 *   FFT forward = exp(-i), inverse = exp(+i), both unnormalised (cuFFT);
 *   parameters that the reference computes in float (windows, ramp phases,
 *   CZT w/a) are computed with the same float expressions; the signal
 *   arithmetic itself (FFTs, sums, products) is carried out in double.
 */
#ifndef ISAR_ORACLE_H_
#define ISAR_ORACLE_H_

#include <complex.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef double _Complex iso_cd;

/* RadarParameters (common.cuh:96-117). */
typedef struct {
    int echo_num;        /* M, pulses (power of two, <= 1024 for parity)   */
    int range_num;       /* N, range cells (power of two, >= 512, >= M)    */
    long long band_width;/* B, Hz                                          */
    long long fc;        /* carrier, Hz                                    */
    double Tp;           /* pulse width, s                                 */
    long long Fs;        /* sampling rate, Hz                              */
} iso_radar;

enum { ISO_IFDS = 1, ISO_STRETCH = 2 };     /* DATA_TYPE, common.cuh:82-87 */

enum {
    ISO_FLAG_HPC  = 1,   /* if_hpc  (isar_main.cu:33)  */
    ISO_FLAG_MTRC = 2,   /* if_mtrc (isar_main.cu:160) */
    ISO_FLAG_HRRP = 4    /* if_hrrp: getHRRP windows STRETCH echoes in place (common.cu:565) */
};

#define ISO_RANGE_NUM_CUT 512           /* common.cuh:71 */
#define ISO_RANGE_NUM_IFDS_PC 4096      /* common.cuh:72 */
#define ISO_ENTROPY_ITERS 120           /* common.cuh:73 */

/* Discrete decisions of one frame, recorded for parity checks. */
typedef struct {
    /* range alignment: one shift per (level, pair): M-1 values, level-major */
    double* ra_shift;          /* caller buffer of M-1 doubles (may be NULL) */
    int     center_applied;    /* 1 if HRRPCenter applied circshiftFreq      */
    int     center_shift;      /* shift_num (range_alignment.cu:457)         */
    float   center_threshold;  /* low_threshold_gray                          */
    int     center_idx1_len, center_idx2_len;
    int     cut_offset;        /* cutRangeProfile offset (common.cu:504-505) */
    int     tgt_num;           /* fastEntropy tgt_num                        */
    int     unit2_num;         /* U = nextPow2(tgt_num/2)                    */
    int     bins[512];         /* selected range bins (sorted), U entries    */
    iso_cd* phase;             /* caller buffer of M: final autofocus phase  */
} iso_trace;

/* ---- primitives -------------------------------------------------------- */
int  iso_next_pow2(int n);                                    /* common.cu:521 */
void iso_hamming_f32(float* w, int len);                      /* common.cu:260 */
/* In-place unnormalised FFT, n a power of two, inverse: sign +. */
int  iso_fft(iso_cd* x, int n, int inverse);
/* Same, on a strided vector (column of a row-major matrix). */
int  iso_fft_strided(iso_cd* x, int n, long stride, int inverse);

/* ---- stages (each in place on double data) ----------------------------- */
void iso_hpc(iso_cd* x, const double* velocity, const iso_radar* p);
void iso_range_align(iso_cd* x, const iso_radar* p, double* shifts);
void iso_hrrp_center(iso_cd* x, const iso_radar* p, int inter_length, iso_trace* tr);
int  iso_cut(const iso_cd* x, iso_cd* cut, int M, int N, int C);
/* getHRRP (common.cu:541-580): M x N range profiles of the echoes. */
void iso_hrrp(const iso_cd* x, iso_cd* out, int M, int N, int data_type);
/* IFDS pulse compression of one pulse (common.cu:583-604, 635-746): 4096
 * complex outputs; returns the cut offset or -1. */
int  iso_pulse_compress(const int16_t* ad, int iq_len, double velocity, const iso_radar* p, iso_cd* out);
void iso_doppler_tracking(iso_cd* comp, iso_cd* phase, const iso_cd* x, int M, int W, int compensate);
void iso_fast_entropy(iso_cd* cut, int M, int C, int iters, iso_trace* tr);
void iso_mtrc(iso_cd* cut, const iso_radar* p, int data_type);
void iso_post(iso_cd* cut, int M, int C, int data_type, double* img);

/*
 * Whole frame, as ISAR_RD_Imaging_Main_Ku (isar_main.cu:3-227) with
 * if_hrrp = false.  echo: interleaved float complex M*N (the reference's
 * d_data_proc); velocity: M doubles (d_velocity, only read with HPC);
 * img: M*512 doubles, |image| row-major [doppler][range].
 * Returns 0, or -1 on invalid sizes.
 */
int iso_image(const float* echo, const double* velocity, const iso_radar* p,
              int data_type, int flags, int iters, double* img, iso_trace* tr);

/* Image entropy -sum p ln p, p = I^2 / sum I^2 (FP64). */
double iso_image_entropy_f32(const float* img, long n);
double iso_image_entropy_f64(const double* img, long n);

/* ---- synthetic dechirped (STRETCH) echoes ------------------------------ */
typedef struct {
    int    M, N;
    double fc, B, prf, Fs;   /* Hz                                         */
    int    n_scat;
    double patch_x, patch_y; /* m, cross-range / range extent of the patch  */
    double omega;            /* rad/s rotation rate                         */
    double r0_cells;         /* bulk range offset of the patch centre, cells */
    double drift_sigma;      /* cells, random-walk step std                 */
    double phase_uniform;    /* rad, half-width of the uniform phase error  */
    double phase_quad;       /* rad, quadratic phase error at the aperture edge */
    double v0, accel;        /* m/s, m/s^2 radial velocity (HPC term)       */
    double snr_db;
    double rms_counts;       /* ADC scale (RMS of the signal part)          */
    uint64_t seed;
} iso_synth_cfg;

/*
 * Fills iq (M*N*2 int16: I,Q interleaved, as the .wbd payload) and
 * velocity (M doubles, quantised to 0.1 m/s like the navigation header).
 */
void iso_synth(const iso_synth_cfg* cfg, int16_t* iq, double* velocity);

#ifdef __cplusplus
}
#endif

#endif /* ISAR_ORACLE_H_ */
