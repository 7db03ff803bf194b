/*
 * isar_oracle.c -- TEST INFRASTRUCTURE ONLY (see isar_oracle.h).
 *
 * FP64 single-threaded restatement of the reference's imaging chain.  Each
 * function names the reference file:line it follows.  Compile with
 * -ffp-contract=off so that the float parameter expressions round exactly as
 * written.
 */
#include "isar_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* Constants exactly as common.cuh:68-70. */
#define PI_FLT 3.14159265358979f
#define PI_DBL 3.14159265358979
#define LIGHT_SPEED 300000000

/* ------------------------------------------------------------------------ */
/* primitives                                                               */
/* ------------------------------------------------------------------------ */

/* nextPow2 (common.cu:521-529): 2^(floor(log2 N)+1); 2N for a power of two. */
int iso_next_pow2(int n)
{
    int r = 1;
    while (n >> 1) {
        r <<= 1;
        n >>= 1;
    }
    return r << 1;
}

/* genHammingVec (common.cu:260-266), float arithmetic as written. */
void iso_hamming_f32(float* w, int len)
{
    for (int i = 0; i < len; ++i) {
        float arg = 2 * PI_FLT * (float)i / (float)(len - 1);
        w[i] = 0.54f - 0.46f * (float)cos((double)arg);
    }
}

static int ilog2i(int n)
{
    int l = 0;
    while ((1 << l) < n) ++l;
    return ((1 << l) == n) ? l : -1;
}

/* Iterative radix-2 DIT FFT with exact double twiddles.  Stands in for cuFFT
 * (the reference's FFTs, common.cu:5-35): same sign and scaling convention. */
int iso_fft_strided(iso_cd* x, int n, long stride, int inverse)
{
    int lg = ilog2i(n);
    if (lg < 0) return -1;
    if (n == 1) return 0;
    /* bit reversal */
    for (int i = 1, j = 0; i < n; ++i) {
        int bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) {
            iso_cd t = x[(long)i * stride];
            x[(long)i * stride] = x[(long)j * stride];
            x[(long)j * stride] = t;
        }
    }
    const double sgn = inverse ? 1.0 : -1.0;
    for (int len = 2; len <= n; len <<= 1) {
        int half = len >> 1;
        for (int k = 0; k < half; ++k) {
            double ang = sgn * 2.0 * M_PI * (double)k / (double)len;
            iso_cd w = cos(ang) + I * sin(ang);
            for (int s = 0; s < n; s += len) {
                iso_cd* a = &x[(long)(s + k) * stride];
                iso_cd* b = &x[(long)(s + k + half) * stride];
                iso_cd t = *b * w;
                *b = *a - t;
                *a = *a + t;
            }
        }
    }
    return 0;
}

int iso_fft(iso_cd* x, int n, int inverse)
{
    return iso_fft_strided(x, n, 1, inverse);
}

/* ifftshiftRows / ifftshiftCols (common.cuh:208-247): swap halves. */
static void shift_rows(iso_cd* x, int rows, int cols)
{
    int h = cols >> 1;
    for (int r = 0; r < rows; ++r) {
        iso_cd* p = x + (long)r * cols;
        for (int i = 0; i < h; ++i) {
            iso_cd t = p[i];
            p[i] = p[i + h];
            p[i + h] = t;
        }
    }
}

static void shift_cols(iso_cd* x, int rows, int cols)
{
    int h = rows >> 1;
    for (int r = 0; r < h; ++r) {
        iso_cd* a = x + (long)r * cols;
        iso_cd* b = x + (long)(r + h) * cols;
        for (int c = 0; c < cols; ++c) {
            iso_cd t = a[c];
            a[c] = b[c];
            b[c] = t;
        }
    }
}

/* Ramp exp(j*val), val = -2*PI_FLT*n*shift/len in float
 * (genFreqMovParallel range_alignment.cu:171-180, genFreqMovVec :361-368). */
static iso_cd ramp_f32(int n, float shift, int len)
{
    float val = -2 * PI_FLT * (float)n * shift / (float)len;
    return cos((double)val) + I * sin((double)val);
}

/* ------------------------------------------------------------------------ */
/* stage 1: high-speed compensation (high_speed_compensation.cu:4-54)        */
/* ------------------------------------------------------------------------ */
void iso_hpc(iso_cd* x, const double* velocity, const iso_radar* p)
{
    const int M = p->echo_num, N = p->range_num;
    const double Fs = (double)p->Fs;
    /* coefficient = -4*pi*K/c  (:17-18) */
    const double chirp_rate = (double)p->band_width / p->Tp;
    const double coef = -4.0 * PI_DBL * chirp_rate / (double)LIGHT_SPEED;
    for (int m = 0; m < M; ++m) {
        for (int n = 0; n < N; ++n) {
            /* genTk2Vec (:57-63), cublasDger into zeroed memory (:32) */
            double tk = (double)n / Fs;
            double ph = coef * (tk * tk) * velocity[m];
            x[(long)m * N + n] *= cos(ph) + I * sin(ph);   /* expJ, multiply */
        }
    }
}

/* ------------------------------------------------------------------------ */
/* stage 2: range alignment (range_alignment.cu:4-78)                        */
/* ------------------------------------------------------------------------ */

/* maxRowsIdxABS tie rule (range_alignment.cu:134-168): per thread class
 * i mod 256 the first maximum; across classes the tree keeps the left
 * operand on ties, i.e. the class with the smallest 8-bit reversed index. */
static int bitrev8(int v)
{
    int r = 0;
    for (int b = 0; b < 8; ++b) r |= ((v >> b) & 1) << (7 - b);
    return r;
}

static int argmax_abs_tree(const double* d, int cols)
{
    int best = -1;
    double bv = 0;
    for (int i = 0; i < cols; ++i) {
        double v = fabs(d[i]);
        if (best < 0 || v > bv) {
            best = i;
            bv = v;
        } else if (v == bv) {
            int ci = i & 255, cb = best & 255;
            if (ci != cb && bitrev8(ci) < bitrev8(cb)) best = i;
        }
    }
    return best;
}

/* binomialFixDevice (range_alignment.cu:121-131), in float as the reference:
 * the correlation sits in a float buffer (d_ave_profile) and the parabola is
 * float arithmetic.  On a broad correlation peak the second difference is
 * tiny, so this rounding moves the shift by up to ~1e-3 cell; keeping it
 * makes the restatement follow the reference instead of the exact value.
 * Neighbours outside the row wrap around (the reference reads the adjacent
 * row there). */
static float binomial_fix(const double* c, int pos, int n)
{
    float f1 = (float)c[(pos - 1 + n) % n];
    float f2 = (float)c[pos];
    float f3 = (float)c[(pos + 1) % n];
    float fa = (f1 + f3 - 2 * f2) / 2;
    float fb = (f3 - f1) / 2;
    return -fb / (2 * fa);
}

/* Circular cross-correlation of two real envelopes as the reference computes
 * it: C2R(R2C(a) * conj(R2C(b))), unnormalised, then ifftshift
 * (range_alignment.cu:50-57). */
static void correlate_shift(const double* a, const double* b, int N, double* corr, iso_cd* wa, iso_cd* wb)
{
    for (int n = 0; n < N; ++n) {
        wa[n] = a[n];
        wb[n] = b[n];
    }
    iso_fft(wa, N, 0);
    iso_fft(wb, N, 0);
    for (int k = 0; k < N; ++k) wa[k] = wa[k] * conj(wb[k]);
    iso_fft(wa, N, 1);
    int h = N >> 1;
    for (int i = 0; i < N; ++i) corr[i] = creal(wa[(i + h) % N]);
}

void iso_range_align(iso_cd* x, const iso_radar* p, double* shifts)
{
    const int M = p->echo_num, N = p->range_num;
    float* ham = (float*)malloc(sizeof(float) * N);
    iso_hamming_f32(ham, N);
    /* genFreqCenteringVec (:195-201) + elementwiseMultiplyRep (:17) */
    for (int n = 0; n < N; ++n) {
        float w = ham[n] * (float)cos((double)(PI_FLT * (float)n));
        for (int m = 0; m < M; ++m) x[(long)m * N + n] *= (double)w;
    }
    free(ham);

    double* prof = (double*)malloc(sizeof(double) * (size_t)M * N);
    double* ave = (double*)malloc(sizeof(double) * (size_t)M * N);
    double* corr = (double*)malloc(sizeof(double) * N);
    iso_cd* tmp = (iso_cd*)malloc(sizeof(iso_cd) * N);
    iso_cd* tmp2 = (iso_cd*)malloc(sizeof(iso_cd) * N);
    int shift_i = 0;

    for (int stride = 1; stride < M; stride *= 2) {
        /* IFFT, 1/N, |.| (:38-42) */
        for (int m = 0; m < M; ++m) {
            memcpy(tmp, x + (long)m * N, sizeof(iso_cd) * N);
            iso_fft(tmp, N, 1);
            for (int n = 0; n < N; ++n) prof[(long)m * N + n] = cabs(tmp[n] / (double)N);
        }
        /* getAveProfileParallel (:81-105): RMS over each group of `stride`
         * rows, stored at the group's first row. */
        for (int g = 0; g < M; g += stride)
            for (int n = 0; n < N; ++n) {
                double s = 0;
                for (int i = 0; i < stride; ++i) {
                    double v = prof[(long)(g + i) * N + n];
                    s += v * v;
                }
                ave[(long)g * N + n] = sqrt(s);
            }
        /* correlation of each pair of heads, argmax, parabolic fix,
         * frequency ramp applied to the second group (:50-69) */
        for (int h1 = 0; h1 < M; h1 += 2 * stride) {
            int h2 = h1 + stride;
            correlate_shift(ave + (long)h1 * N, ave + (long)h2 * N, N, corr, tmp, tmp2);
            int pos = argmax_abs_tree(corr, N);
            float shf = (float)pos + binomial_fix(corr, pos, N) - ((float)N / 2);   /* :166 */
            if (shifts) shifts[shift_i] = shf;
            ++shift_i;
            for (int n = 0; n < N; ++n) {
                iso_cd r = ramp_f32(n, shf, N);
                for (int m = h2; m < h2 + stride; ++m) x[(long)m * N + n] *= r;
            }
        }
    }
    /* final IFFT, 1/N (:76-77) */
    for (int m = 0; m < M; ++m) {
        iso_fft(x + (long)m * N, N, 1);
        for (int n = 0; n < N; ++n) x[(long)m * N + n] /= (double)N;
    }
    free(prof);
    free(ave);
    free(corr);
    free(tmp);
    free(tmp2);
}

/* ------------------------------------------------------------------------ */
/* HRRPCenter (range_alignment.cu:371-465)                                   */
/* ------------------------------------------------------------------------ */

static int cmp_double(const void* a, const void* b)
{
    double x = *(const double*)a, y = *(const double*)b;
    return (x > y) - (x < y);
}

/* getARPMean (range_alignment.cu:524-550), including its edge divisors. */
static double arp_mean(const double* arp, int idx, int WL, int N)
{
    double s = 0;
    if (idx - WL / 2 >= 0 && idx + WL / 2 <= N - 1) {
        for (int i = idx - WL / 2; i <= idx + WL / 2; ++i) s += arp[i];
        s /= (double)(WL + 1);
    } else if (idx - WL / 2 < 0) {
        for (int i = 0; i <= idx + WL / 2; ++i) s += arp[i];
        s /= ((double)WL / 2 + idx + 1);
    } else if (idx + WL / 2 > N - 1) {
        for (int i = idx - WL / 2; i < N; ++i) s += arp[i];
        s /= ((double)N - idx - ((double)WL / 2) - 1);
    }
    return s;
}

void iso_hrrp_center(iso_cd* x, const iso_radar* p, int inter_length, iso_trace* tr)
{
    const int M = p->echo_num, N = p->range_num;
    /* |x| / max|x| (:380-389) */
    double hmax = 0;
    for (long i = 0; i < (long)M * N; ++i) {
        double a = cabs(x[i]);
        if (a > hmax) hmax = a;
    }
    /* ARP = sum over the first 256 rows (sumCols launched with 256 threads,
     * :396) times 1/M (:398-399); rows [0, min(M,256)). */
    int rows = M < 256 ? M : 256;
    double* arp = (double*)calloc(N, sizeof(double));
    for (int n = 0; n < N; ++n) {
        double s = 0;
        for (int m = 0; m < rows; ++m) s += cabs(x[(long)m * N + n]) / hmax;
        arp[n] = s * (1.0 / (double)M);
    }
    /* noise threshold (:402-423) */
    double* arp1 = (double*)malloc(sizeof(double) * N);
    memcpy(arp1, arp, sizeof(double) * N);
    qsort(arp1, N, sizeof(double), cmp_double);
    double arp1_max = 0;
    for (int i = 0; i < N; ++i)
        if (fabs(arp1[i]) > fabs(arp1_max)) arp1_max = arp1[i];
    double extra = (double)inter_length * arp1_max / (double)N;
    int diff_len = N - inter_length;
    int dmin = 0;
    double dmin_v = 0;
    for (int i = 0; i < diff_len; ++i) {
        double d = fabs(arp1[i + inter_length] - arp1[i] - extra);
        if (i == 0 || d < dmin_v) {
            dmin = i;
            dmin_v = d;
        }
    }
    double thr = arp1[dmin + inter_length / 2];
    /* idx_1 = find(arp > thr), windowed means, idx_2 = find(mean < thr) (:426-449) */
    int* idx1 = (int*)malloc(sizeof(int) * N);
    int n1 = 0;
    for (int n = 0; n < N; ++n)
        if (arp[n] > thr) idx1[n1++] = n;
    int n2 = 0;
    long sum = 0;
    const int WL = 8;
    for (int t = 0; t < n1; ++t) {
        if (arp_mean(arp, idx1[t], WL, N) < thr)
            ++n2;
        else
            sum += idx1[t];
    }
    int applied = 0, shift_num = 0;
    if (n2 != n1) {
        /* (:451-460): integer mean index, circshiftFreq by N/2 - mean */
        int mean_idx = (int)(sum / (long)(n1 - n2));
        shift_num = -(mean_idx - N / 2);
        applied = 1;
        iso_cd* row = (iso_cd*)malloc(sizeof(iso_cd) * N);
        /* circshiftFreq (:496-521): FFT, ramp (float phase), IFFT, 1/N */
        for (int m = 0; m < M; ++m) {
            memcpy(row, x + (long)m * N, sizeof(iso_cd) * N);
            iso_fft(row, N, 0);
            for (int n = 0; n < N; ++n) row[n] *= ramp_f32(n, (float)shift_num, N);
            iso_fft(row, N, 1);
            for (int n = 0; n < N; ++n) x[(long)m * N + n] = row[n] / (double)N;
        }
        free(row);
    }
    if (tr) {
        tr->center_applied = applied;
        tr->center_shift = shift_num;
        tr->center_threshold = (float)thr;
        tr->center_idx1_len = n1;
        tr->center_idx2_len = n2;
    }
    free(arp);
    free(arp1);
    free(idx1);
}

/* cutRangeProfile (common.cu:494-509): cublasIcamax (|Re|+|Im|, first
 * maximum) on row 0, offset = clamp(idx - C/2, 0, N - C), gather. */
int iso_cut(const iso_cd* x, iso_cd* cut, int M, int N, int C)
{
    int idx = 0;
    double bv = -1;
    for (int n = 0; n < N; ++n) {
        double v = fabs(creal(x[n])) + fabs(cimag(x[n]));
        if (v > bv) {
            bv = v;
            idx = n;
        }
    }
    int off = idx - C / 2;
    if (off < 0) off = 0;
    if (off > N - C) off = N - C;
    for (int m = 0; m < M; ++m)
        memcpy(cut + (long)m * C, x + (long)m * N + off, sizeof(iso_cd) * C);
    return off;
}

/* getHRRP (common.cu:541-580), the high-resolution range profiles of a
 * frame: STRETCH: row-wise FFT of the echoes times the float range Hamming
 * window (genHammingVec over N, which the reference applies in place),
 * then ifftshiftRows; IFDS: ifftshiftRows, FFT, ifftshiftRows.  Rows of N
 * (even: the shift swaps the halves). */
void iso_hrrp(const iso_cd* x, iso_cd* out, int M, int N, int data_type)
{
    float* ham = (float*)malloc(sizeof(float) * (size_t)N);
    iso_cd* row = (iso_cd*)malloc(sizeof(iso_cd) * (size_t)N);
    iso_hamming_f32(ham, N);
    const int h = N / 2;
    for (int m = 0; m < M; ++m) {
        const iso_cd* xr = x + (size_t)m * N;
        for (int n = 0; n < N; ++n)
            row[n] = data_type == ISO_STRETCH ? xr[n] * (double)ham[n] : xr[(n + h) % N];
        iso_fft(row, N, 0);
        for (int n = 0; n < N; ++n) out[(size_t)m * N + n] = row[(n + h) % N];
    }
    free(ham);
    free(row);
}

/* ------------------------------------------------------------------------ */
/* IFDS ingest: per-pulse matched-filter pulse compression                   */
/* ------------------------------------------------------------------------ */

/* pulseCompression::pulseCompressionbyFFT (common.cu:635-746) for one pulse,
 * as multiThreadIFDS drives it (common.cu:583-604): ad holds 2*iq_len int16
 * samples (I, Q interleaved; common.cu:597-599), NFFT = nextPow2(iq_len)
 * (Q8: 2*iq_len for a power of two), S = (int)(Fs * Tp) reference samples.
 * Reference chirp (genTkPulseCompression, genRefPulseCompression,
 * common.cu:620-660): tk = (1 - v2)(-Tp/2 + i Tp/(S-1)),
 * ref = hamming_S[i] exp(j (c1 + c2 tk) tk), c1 = -2 pi fc v2/(1 - v2),
 * c2 = pi B / Tp, v2 = 2 v / c, all in float as written (no contraction).
 * y = IFFT(conj(FFT(ref)) .* FFT(x)) / NFFT (elementwiseMultiplyConjA,
 * cublasCsscal), then cutRangeProfile with one row (common.cu:494-509):
 * Icamax (|Re|+|Im|, first maximum), offset = clamp(idx - 2048, 0, NFFT - 4096),
 * out = y[offset .. offset + 4096).  Signal arithmetic in double.
 * Returns the offset, or -1 when NFFT < 4096 or S outside [2, NFFT]. */
int iso_pulse_compress(const int16_t* ad, int iq_len, double velocity, const iso_radar* p, iso_cd* out)
{
    const int nfft = iso_next_pow2(iq_len);
    const int S = (int)((double)p->Fs * p->Tp);
    if (nfft < ISO_RANGE_NUM_IFDS_PC || S < 2 || S > nfft) return -1;
    iso_cd* x = (iso_cd*)calloc((size_t)nfft, sizeof(iso_cd));
    iso_cd* r = (iso_cd*)calloc((size_t)nfft, sizeof(iso_cd));
    float* ham = (float*)malloc(sizeof(float) * (size_t)S);
    for (int i = 0; i < iq_len; ++i) x[i] = (double)ad[2 * i] + I * (double)ad[2 * i + 1];
    const float v2 = 2 * (float)velocity / (float)LIGHT_SPEED;
    const float v2c = 1 - v2;
    const float c1 = -2 * PI_FLT * (float)p->fc * v2 / v2c;
    const float c2 = (float)((double)(PI_FLT * (float)p->band_width) / p->Tp);
    const float tpf = (float)p->Tp;
    iso_hamming_f32(ham, S);
    for (int i = 0; i < S; ++i) {
        const float tk = v2c * (tpf / -2.0f + (float)i * tpf / ((float)S - 1.0f));
        const float ph = (c1 + c2 * tk) * tk;
        const float cr = ham[i] * (float)cos((double)ph), ci = ham[i] * (float)sin((double)ph);
        r[i] = (double)cr + I * (double)ci;
    }
    iso_fft(x, nfft, 0);
    iso_fft(r, nfft, 0);
    for (int k = 0; k < nfft; ++k) x[k] = conj(r[k]) * x[k];
    iso_fft(x, nfft, 1);
    const double sc = 1.0 / nfft;
    int idx = 0;
    double bv = -1;
    for (int n = 0; n < nfft; ++n) {
        x[n] *= sc;
        const double v = fabs(creal(x[n])) + fabs(cimag(x[n]));
        if (v > bv) {
            bv = v;
            idx = n;
        }
    }
    int off = idx - ISO_RANGE_NUM_IFDS_PC / 2;
    if (off < 0) off = 0;
    if (off > nfft - ISO_RANGE_NUM_IFDS_PC) off = nfft - ISO_RANGE_NUM_IFDS_PC;
    memcpy(out, x + off, sizeof(iso_cd) * ISO_RANGE_NUM_IFDS_PC);
    free(x);
    free(r);
    free(ham);
    return off;
}

/* ------------------------------------------------------------------------ */
/* stage 3/4: Doppler tracking + fast entropy (phase_adjustment.cu)          */
/* ------------------------------------------------------------------------ */

/* dopplerTracking (phase_adjustment.cu:4-41).  phase[0] = 0 (Q2). */
void iso_doppler_tracking(iso_cd* comp, iso_cd* phase, const iso_cd* x, int M, int W, int compensate)
{
    double acc = 0;
    phase[0] = 0;
    for (int m = 0; m < M - 1; ++m) {
        iso_cd s = 0;
        for (int c = 0; c < W; ++c) s += conj(x[(long)m * W + c]) * x[(long)(m + 1) * W + c];
        acc += carg(s);                       /* inclusive_scan of arg  */
        phase[m + 1] = cos(acc) - I * sin(acc);  /* exp(-j*angle)         */
    }
    if (compensate)
        for (int m = 0; m < M; ++m)
            for (int c = 0; c < W; ++c) comp[(long)m * W + c] = phase[m] * x[(long)m * W + c];
}

typedef struct {
    double key;
    int idx;
} kv_t;

static int cmp_kv_desc(const void* a, const void* b)
{
    const kv_t* x = (const kv_t*)a;
    const kv_t* y = (const kv_t*)b;
    if (x->key > y->key) return -1;
    if (x->key < y->key) return 1;
    return (x->idx > y->idx) - (x->idx < y->idx);   /* stable */
}

/* stable ascending by key; ties keep the current order, carried in pos */
typedef struct {
    double key;
    int pos;
    int idx;
} kv3_t;

static int cmp_kv3_asc(const void* a, const void* b)
{
    const kv3_t* x = (const kv3_t*)a;
    const kv3_t* y = (const kv3_t*)b;
    if (x->key < y->key) return -1;
    if (x->key > y->key) return 1;
    return (x->pos > y->pos) - (x->pos < y->pos);
}

static int cmp_int(const void* a, const void* b)
{
    int x = *(const int*)a, y = *(const int*)b;
    return (x > y) - (x < y);
}

/* fastEntropy (phase_adjustment.cu:167-332) */
void iso_fast_entropy(iso_cd* cut, int M, int C, int iters, iso_trace* tr)
{
    const long MC = (long)M * C;
    /* colmax of |x| over the first 256 rows (maxCols, 256 threads, :183) */
    int rows = M < 256 ? M : 256;
    double* colmax = (double*)malloc(sizeof(double) * C);
    for (int c = 0; c < C; ++c) {
        double mx = cabs(cut[c]);
        for (int m = 1; m < rows; ++m) {
            double a = cabs(cut[(long)m * C + c]);
            if (a > mx) mx = a;
        }
        colmax[c] = mx;
    }
    /* mean with an int accumulator (Q3, :187), threshold 1.48*mean */
    long long isum = 0;
    for (int c = 0; c < C; ++c) isum += (int)colmax[c];
    float mean_val = (float)(int)isum / (float)C;
    float threshold = 1.48f * mean_val;
    int tgt_num = 0;
    for (int c = 0; c < C; ++c)
        if (colmax[c] > (double)threshold) ++tgt_num;

    /* Doppler-compensated copy, column FFT, energy and entropy (:198-246) */
    iso_cd* comp = (iso_cd*)malloc(sizeof(iso_cd) * MC);
    iso_cd* phase = (iso_cd*)malloc(sizeof(iso_cd) * M);
    iso_doppler_tracking(comp, phase, cut, M, C, 1);
    for (int c = 0; c < C; ++c) iso_fft_strided(comp + c, M, C, 0);
    double* energy = (double*)malloc(sizeof(double) * C);
    double* ent = (double*)malloc(sizeof(double) * C);
    for (int c = 0; c < C; ++c) {
        double e = 0;
        for (int m = 0; m < M; ++m) {
            double a = cabs(comp[(long)m * C + c]);
            e += a * a;
        }
        double h = 0;
        for (int m = 0; m < M; ++m) {
            double a = cabs(comp[(long)m * C + c]);
            double q = a * a / e;
            h += -(q * log(q));
        }
        energy[c] = e;
        ent[c] = h;
    }
    /* top tgt_num by energy (stable, descending), then the U lowest entropy
     * (stable), then sorted indices (:249-264) */
    int U = iso_next_pow2(tgt_num / 2);
    kv_t* ke = (kv_t*)malloc(sizeof(kv_t) * C);
    for (int c = 0; c < C; ++c) {
        ke[c].key = energy[c];
        ke[c].idx = c;
    }
    qsort(ke, C, sizeof(kv_t), cmp_kv_desc);
    kv3_t* kh = (kv3_t*)malloc(sizeof(kv3_t) * (tgt_num > 0 ? tgt_num : 1));
    for (int i = 0; i < tgt_num; ++i) {
        kh[i].key = ent[ke[i].idx];
        kh[i].pos = i;
        kh[i].idx = ke[i].idx;
    }
    qsort(kh, tgt_num, sizeof(kv3_t), cmp_kv3_asc);
    int bins[512];
    for (int u = 0; u < U; ++u) bins[u] = (u < tgt_num) ? kh[u].idx : 0;   /* resize pads 0 */
    qsort(bins, U, sizeof(int), cmp_int);

    /* g = selected range bins, phase from Doppler tracking (:266-282) */
    iso_cd* g = (iso_cd*)malloc(sizeof(iso_cd) * (size_t)M * U);
    for (int m = 0; m < M; ++m)
        for (int u = 0; u < U; ++u) g[(long)m * U + u] = cut[(long)m * C + bins[u]];
    iso_doppler_tracking(NULL, phase, g, M, U, 0);

    /* minimum-entropy iterations (:302-322) */
    iso_cd* t = (iso_cd*)malloc(sizeof(iso_cd) * (size_t)M * U);
    for (int it = 0; it < iters; ++it) {
        for (int m = 0; m < M; ++m)
            for (int u = 0; u < U; ++u) t[(long)m * U + u] = phase[m] * g[(long)m * U + u];
        for (int u = 0; u < U; ++u) {
            iso_fft_strided(t + u, M, U, 0);
            for (int m = 0; m < M; ++m) {
                iso_cd v = t[(long)m * U + u];
                t[(long)m * U + u] = v * cabs(v);
            }
            iso_fft_strided(t + u, M, U, 1);
        }
        for (int m = 0; m < M; ++m) {
            iso_cd s = 0;
            for (int u = 0; u < U; ++u)
                s += conj(g[(long)m * U + u]) * (t[(long)m * U + u] * (1.0 / (double)M));
            phase[m] = s / cabs(s);
        }
    }
    /* apply to the whole cut (:324) */
    for (int m = 0; m < M; ++m)
        for (int c = 0; c < C; ++c) cut[(long)m * C + c] *= phase[m];

    if (tr) {
        tr->tgt_num = tgt_num;
        tr->unit2_num = U;
        for (int u = 0; u < U && u < 512; ++u) tr->bins[u] = bins[u];
        if (tr->phase) memcpy(tr->phase, phase, sizeof(iso_cd) * M);
    }
    free(colmax);
    free(comp);
    free(phase);
    free(energy);
    free(ent);
    free(ke);
    free(kh);
    free(g);
    free(t);
}

/* ------------------------------------------------------------------------ */
/* stage 5: MTRC (mtrc.cu:4-192)                                             */
/* ------------------------------------------------------------------------ */

/* complex power of a float-valued complex number, exp(y * log(z)), the
 * formula thrust::pow uses (mtrc.cu:87,102); evaluated in double. */
static iso_cd cpow_f32base(float re, float im, double y)
{
    double lr = 0.5 * log1p(((double)re - 1.0) * ((double)re + 1.0) + (double)im * (double)im);
    double th = atan2((double)im, (double)re);
    double mag = exp(y * lr);
    double ang = y * th;
    return mag * cos(ang) + I * mag * sin(ang);
}

/* getWandA (mtrc.cu:175-192): float parameters.  The inner sum
 * 1 - constant + posa*n is formed with one fused multiply-add, as the CUDA
 * compiler contracts it. */
static void mtrc_wa(const iso_radar* p, int C, float* wre, float* wim, float* are, float* aim)
{
    const int M = p->echo_num;
    float chirp_rate = (float)p->band_width / (float)p->Tp;                       /* :10 */
    float posa = chirp_rate * (float)p->Tp / ((float)p->fc * ((float)C - 1.0f));   /* :12 */
    float constant = chirp_rate * (float)p->Tp / (float)(2 * p->fc);              /* :47 */
    for (int c = 0; c < C; ++c) {
        float base = fmaf(posa, (float)c, 1 - constant);
        float tw = -2 * PI_FLT * base / (float)M;
        float ta = -1 * PI_FLT * base;
        wre[c] = (float)cos((double)tw);
        wim[c] = (float)sin((double)tw);
        are[c] = (float)cos((double)ta);
        aim[c] = (float)sin((double)ta);
    }
}

void iso_mtrc(iso_cd* cut, const iso_radar* p, int data_type)
{
    const int M = p->echo_num, C = ISO_RANGE_NUM_CUT;
    const long MC = (long)M * C;
    iso_cd* st = (iso_cd*)malloc(sizeof(iso_cd) * MC);
    memcpy(st, cut, sizeof(iso_cd) * MC);
    /* ifftshift rows, row IFFT/C (STRETCH) or FFT (IFDS) (:18-40) */
    shift_rows(st, M, C);
    for (int m = 0; m < M; ++m) {
        if (data_type == ISO_IFDS) {
            iso_fft(st + (long)m * C, C, 0);
        } else {
            iso_fft(st + (long)m * C, C, 1);
            for (int c = 0; c < C; ++c) st[(long)m * C + c] /= (double)C;
        }
    }
    float *wre = (float*)malloc(sizeof(float) * C * 4);
    float *wim = wre + C, *are = wre + 2 * C, *aim = wre + 3 * C;
    mtrc_wa(p, C, wre, wim, are, aim);

    /* cztRange (:125-172), Bluestein with L = nextPow2(2M-1) */
    const int L = iso_next_pow2(2 * M - 1);
    const int wwl = 2 * M - 1;
    iso_cd* ww = (iso_cd*)malloc(sizeof(iso_cd) * wwl);
    iso_cd* y = (iso_cd*)malloc(sizeof(iso_cd) * L);
    iso_cd* v = (iso_cd*)malloc(sizeof(iso_cd) * L);
    for (int c = 0; c < C; ++c) {
        for (int k = 0; k < wwl; ++k) {      /* genWW (:79-93) */
            int kk = k - (M - 1);
            float kk2 = (float)(kk * kk) / 2.0f;
            ww[k] = cpow_f32base(wre[c], wim[c], (double)kk2);
        }
        for (int k = 0; k < L; ++k) {        /* gety (:96-109) */
            if (k < M)
                y[k] = cpow_f32base(are[c], aim[c], -(double)k) * ww[M - 1 + k] * st[(long)k * C + c];
            else
                y[k] = 0;
            v[k] = (k < wwl) ? 1.0 / ww[k] : 0;   /* pow(ww,-1), zero tail (Q4) */
        }
        iso_fft(y, L, 0);
        iso_fft(v, L, 0);
        for (int k = 0; k < L; ++k) y[k] *= v[k];
        iso_fft(y, L, 1);
        for (int k = 0; k < M; ++k)          /* getCZTOut (:112-122) */
            cut[(long)k * C + c] = (y[M - 1 + k] / (double)L) * ww[M - 1 + k];
    }
    /* column ifftshift, column IFFT/M, column ifftshift, row FFT,
     * row fftshift, column fftshift (:53-70) */
    shift_cols(cut, M, C);
    for (int c = 0; c < C; ++c) iso_fft_strided(cut + c, M, C, 1);
    for (long i = 0; i < MC; ++i) cut[i] /= (double)M;
    shift_cols(cut, M, C);
    for (int m = 0; m < M; ++m) iso_fft(cut + (long)m * C, C, 0);
    shift_rows(cut, M, C);
    shift_cols(cut, M, C);
    if (data_type == ISO_IFDS) {             /* fliplr (:72-75) */
        for (int m = 0; m < M; ++m)
            for (int c = 0; c < C / 2; ++c) {
                iso_cd t = cut[(long)m * C + c];
                cut[(long)m * C + c] = cut[(long)m * C + C - 1 - c];
                cut[(long)m * C + C - 1 - c] = t;
            }
    }
    free(st);
    free(wre);
    free(ww);
    free(y);
    free(v);
}

/* post-processing (isar_main.cu:191-211): Hamming over pulses, column FFT,
 * column fftshift, (IFDS: flipud), |.|.
 * The window launch (isar_main.cu:192) passes cols = echo_num and
 * len = range_num_cut to diagMulMat(diag, data, res, cols, len)
 * (common.cu:230-238), so it only touches the first 512 elements:
 * element i < 512 (row 0) is scaled by hamming[i / echo_num] and every other
 * row is left unwindowed (Q13).  Reproduced as the reference computes it. */
void iso_post(iso_cd* cut, int M, int C, int data_type, double* img)
{
    float* hm = (float*)malloc(sizeof(float) * M);
    iso_hamming_f32(hm, M);
    for (int i = 0; i < ISO_RANGE_NUM_CUT && i < M * C; ++i) cut[i] *= (double)hm[i / M];
    free(hm);
    for (int c = 0; c < C; ++c) iso_fft_strided(cut + c, M, C, 0);
    shift_cols(cut, M, C);
    if (data_type == ISO_IFDS) {
        for (int m = 0; m < M / 2; ++m)
            for (int c = 0; c < C; ++c) {
                iso_cd t = cut[(long)m * C + c];
                cut[(long)m * C + c] = cut[(long)(M - 1 - m) * C + c];
                cut[(long)(M - 1 - m) * C + c] = t;
            }
    }
    for (long i = 0; i < (long)M * C; ++i) img[i] = cabs(cut[i]);
}

/* ------------------------------------------------------------------------ */
/* whole frame: ISAR_RD_Imaging_Main_Ku (isar_main.cu:3-227)                 */
/* ------------------------------------------------------------------------ */
int iso_image(const float* echo, const double* velocity, const iso_radar* p,
              int data_type, int flags, int iters, double* img, iso_trace* tr)
{
    const int M = p->echo_num, N = p->range_num, C = ISO_RANGE_NUM_CUT;
    if (M < 2 || N < C || N < M || ilog2i(M) < 0 || ilog2i(N) < 0) return -1;
    iso_cd* x = (iso_cd*)malloc(sizeof(iso_cd) * (size_t)M * N);
    iso_cd* cut = (iso_cd*)malloc(sizeof(iso_cd) * (size_t)M * C);
    if (!x || !cut) {
        free(x);
        free(cut);
        return -2;
    }
    for (long i = 0; i < (long)M * N; ++i) x[i] = (double)echo[2 * i] + I * (double)echo[2 * i + 1];

    if (data_type == ISO_IFDS) {            /* isar_main.cu:15-27 */
        shift_rows(x, M, N);
        for (int m = 0; m < M; ++m) {
            iso_fft(x + (long)m * N, N, 1);
            for (int n = 0; n < N; ++n) x[(long)m * N + n] /= (double)N;
        }
        shift_rows(x, M, N);
    }
    if ((flags & ISO_FLAG_HPC) && data_type == ISO_STRETCH) iso_hpc(x, velocity, p);
    if ((flags & ISO_FLAG_HRRP) && data_type == ISO_STRETCH) {
        /* getHRRP (common.cu:563-566): x *= hamming(n) in place; the HRRP
         * itself is never returned by the reference */
        float* ham = (float*)malloc(sizeof(float) * N);
        iso_hamming_f32(ham, N);
        for (int m = 0; m < M; ++m)
            for (int n = 0; n < N; ++n) x[(long)m * N + n] *= (double)ham[n];
        free(ham);
    }
    iso_range_align(x, p, tr ? tr->ra_shift : NULL);
    iso_hrrp_center(x, p, 30, tr);                          /* inter_length = 30 */
    int off = iso_cut(x, cut, M, N, C);
    if (tr) tr->cut_offset = off;
    iso_fast_entropy(cut, M, C, iters, tr);
    if (flags & ISO_FLAG_MTRC) iso_mtrc(cut, p, data_type);
    iso_post(cut, M, C, data_type, img);
    free(x);
    free(cut);
    return 0;
}

double iso_image_entropy_f64(const double* img, long n)
{
    double s = 0;
    for (long i = 0; i < n; ++i) s += img[i] * img[i];
    double e = 0;
    for (long i = 0; i < n; ++i) {
        double q = img[i] * img[i] / s;
        if (q > 0) e -= q * log(q);
    }
    return e;
}

double iso_image_entropy_f32(const float* img, long n)
{
    double s = 0;
    for (long i = 0; i < n; ++i) s += (double)img[i] * img[i];
    double e = 0;
    for (long i = 0; i < n; ++i) {
        double q = (double)img[i] * img[i] / s;
        if (q > 0) e -= q * log(q);
    }
    return e;
}

/* ------------------------------------------------------------------------ */
/* synthetic dechirped echoes                                               */
/* ------------------------------------------------------------------------ */
static uint64_t sm_next(uint64_t* s)
{
    uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static double sm_uniform(uint64_t* s)   /* (0,1) */
{
    return ((double)(sm_next(s) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

static double sm_gauss(uint64_t* s)
{
    double u1 = sm_uniform(s), u2 = sm_uniform(s);
    return sqrt(-2.0 * log(u1)) * cos(2.0 * M_PI * u2);
}

void iso_synth(const iso_synth_cfg* cfg, int16_t* iq, double* velocity)
{
    const int M = cfg->M, N = cfg->N, K = cfg->n_scat;
    const double c = (double)LIGHT_SPEED;
    const double Tp = (double)N / cfg->Fs;
    const double Kr = cfg->B / Tp;
    const double cell = c / (2.0 * cfg->B);
    uint64_t s = cfg->seed;
    double* sx = (double*)malloc(sizeof(double) * K * 4);
    double *sy = sx + K, *amp = sx + 2 * K, *ph0 = sx + 3 * K;
    double pw = 0;
    for (int k = 0; k < K; ++k) {
        sx[k] = (sm_uniform(&s) - 0.5) * cfg->patch_x;
        sy[k] = (sm_uniform(&s) - 0.5) * cfg->patch_y;
        amp[k] = sqrt(-2.0 * log(sm_uniform(&s)));     /* Rayleigh */
        ph0[k] = 2.0 * M_PI * sm_uniform(&s);
        pw += amp[k] * amp[k];
    }
    double* drift = (double*)malloc(sizeof(double) * M * 3);
    double *perr = drift + M, *vel = drift + 2 * M;
    double d = 0;
    for (int m = 0; m < M; ++m) {
        drift[m] = d * cell;
        d += cfg->drift_sigma * sm_gauss(&s);
        double u = (double)(m - M / 2) / (double)(M / 2);
        perr[m] = cfg->phase_quad * u * u + cfg->phase_uniform * (2.0 * sm_uniform(&s) - 1.0);
        vel[m] = cfg->v0 + cfg->accel * (double)m / cfg->prf;
        /* navigation header: signed 0.1 m/s (common.cu:871-875) */
        velocity[m] = (double)llround(vel[m] * 10.0) * 0.1;
    }
    double scale = cfg->rms_counts / sqrt(pw > 0 ? pw : 1.0);
    double nsig = sqrt(pw / pow(10.0, cfg->snr_db / 10.0) / 2.0);
    for (int m = 0; m < M; ++m) {
        double th = cfg->omega * (double)(m - M / 2) / cfg->prf;
        double ct = cos(th), st = sin(th);
        for (int n = 0; n < N; ++n) {
            double t = (double)n / cfg->Fs;
            double f = cfg->fc + Kr * t;
            double re = 0, im = 0;
            for (int k = 0; k < K; ++k) {
                double R = cfg->r0_cells * cell + drift[m] + sy[k] * ct + sx[k] * st;
                double ph = -(4.0 * M_PI / c) * f * (R - vel[m] * t) + perr[m] + ph0[k];
                re += amp[k] * cos(ph);
                im += amp[k] * sin(ph);
            }
            re += nsig * sm_gauss(&s);
            im += nsig * sm_gauss(&s);
            double vr = nearbyint(re * scale), vi = nearbyint(im * scale);
            if (vr > 32767) vr = 32767;
            if (vr < -32768) vr = -32768;
            if (vi > 32767) vi = 32767;
            if (vi < -32768) vi = -32768;
            iq[2 * ((long)m * N + n)] = (int16_t)vr;
            iq[2 * ((long)m * N + n) + 1] = (int16_t)vi;
        }
    }
    free(sx);
    free(drift);
}
