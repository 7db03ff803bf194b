// Internal launcher interface between the host pipeline and the kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <mutex>

namespace isar {

namespace nn {
struct Weights;
struct Acts;
}  // namespace nn

// Number of kernels this library has launched (all contexts).
inline std::atomic<long long>& launch_counter()
{
    static std::atomic<long long> n{0};
    return n;
}
#define ISAR_COUNT(n) (::isar::launch_counter() += (n))

// One value per device ordinal, computed once per device by a set-up function
// run with that device current (kernel attributes, occupancy queries: both
// are per device).  Thread-safe; a negative result (an error) is returned
// but not kept, so the next call retries.  Devices beyond kSlots are set up
// on every call.
class PerDevice {
  public:
    PerDevice()
    {
        for (auto& v : val_) v.store(kUnset, std::memory_order_relaxed);
    }
    template <class F>
    int get(F&& setup)
    {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kSlots) {
            (void)cudaGetLastError();
            return setup();
        }
        int v = val_[dev].load(std::memory_order_acquire);
        if (v != kUnset) return v;
        std::lock_guard<std::mutex> lock(mu_);
        v = val_[dev].load(std::memory_order_relaxed);
        if (v != kUnset) return v;
        v = setup();
        if (v >= 0) val_[dev].store(v, std::memory_order_release);
        return v;
    }

  private:
    static constexpr int kSlots = 64;
    static constexpr int kUnset = -0x7fffffff;
    std::atomic<int> val_[kSlots];
    std::mutex mu_;
};

struct RAArgs {
    int M, N;
    const float2* x;         // [M][N] spectra in
    float2* y;               // [M][N] range profiles out (may equal x)
    const float* win;        // [N] hamming(n) * cos(pi*n), float as the reference
    const int64_t* hq;       // [M] HPC phase coefficient (fixed point) or nullptr
    double* S;               // [M] cumulative alignment shift, cells
    int64_t* SQ;             // [M] S / N as a 64-bit fixed-point fraction of a cycle
    float* shifts;           // [M-1] per (level, pair) shift, level-major
    float* env_a;            // [M][N] envelope ping buffer; merged spectra [M/2][N] complex
    float* env_b;            // [M/2][N] envelope pong buffer (may lie inside env_a's second half)
    float* part;             // [max(M/2,256)][N] partial sums; merged spectra [M/4][N] complex
    float* arp;              // [N] average range profile
    unsigned* hmax;          // max |y| (float bits)
    const float2* tw;        // twiddle table exp(-2 pi i k / kTwN)
    int rows_each_level;     // 1: transform the shifted rows at every level (carried
                             // envelopes); 0: spectral envelope merge
    int pair_min;            // use the fused pair kernel while pairs >= pair_min
    int rpc;                 // rows per CTA for the accumulate kernel
    int rpc_final;           // rows per CTA for the final transform
    int given_shifts;        // use the shifts already in `shifts` (test hook)
    unsigned* err;           // set when a row-copy wait runs out (rows invalid)
    int x_iq16;              // x holds int16 I/Q pairs (level 0 reads them directly)
};

// Poll limit of the autofocus grid barrier (about a second of polling), and
// the test hook that makes it run out: `extra` arrivals are added to every
// barrier's target, so no CTA can pass and each gives up after `limit` polls.
constexpr unsigned long long kSpinLimit = 1ull << 22;
struct BarrierTest {
    unsigned long long limit = kSpinLimit;
    unsigned extra = 0;
};

struct FEArgs {
    int M;
    int iters;
    float2* cut;             // [M][512], phase applied in place at the end
    float* cmax_part;        // [ceil(min(M,256)/8)][512]
    float2* dsum;            // [M]
    float2* phase;           // [M]
    int* fdec;               // [0] tgt_num, [1] U
    double* E;               // [512]
    double* H;               // [512]
    int* bins;               // [512]
    float2* sig_part;        // [M][128] autofocus partial row sums
    float2* gcol;            // [512][M] gathered bin columns (cluster engine, M = 1024)
    unsigned* bar;           // [0] grid-barrier counter, [1] barrier timeout flag
    BarrierTest bar_test;    // poll limit and target offset of the grid barrier
    const float2* tw;
    // Autofocus engine: 0 = one cooperative grid (128 CTAs, grid barriers);
    // 4, 8 or 16 = one thread-block cluster of that many CTAs per frame
    // (distributed shared memory, no grid barrier).
    int af_cluster;
    // Entropy stop criterion (cluster engine): stop once the entropy of the
    // selected bins changes by <= tol * |entropy| per iteration (mean over
    // the 4 iterations between two checks); 0 runs all `iters` (the
    // reference's fixed count).
    float tol;
    int* af_stat;            // [0] iterations applied (both legs with a warm start), [1] entropy
                             // (float bits), [2] learned leg kept (set by the image judge),
                             // [3], [4] entropies of the plain and learned legs (float bits),
                             // [5], [6] their iterations; may be null
    // Learned warm start (cluster engine only), or ws_w == nullptr.
    const nn::Weights* ws_w;
    nn::Acts* ws_a;          // inference activations for M rows; act[0] receives the features
    float* ws_psi;           // [M]
    float2* ws_phase;        // [M] warm-start phase in, the learned leg's final phase out
    float2* cut2;            // [M][512] the learned leg's phase applied to the cut (warm start;
                             // not written with defer_apply, where the imaging applies it)
    int* ws_err;             // GEMM wait-timeout flag
    int pre_only;            // stop after the bin selection and the Doppler start phase
    int defer_apply;         // leave the cut unphased: the imaging applies the phase(s)
                             // (PostArgs::phase; MTRC at M >= 512 only)
};

// Largest cluster the device accepts for the autofocus engine with M pulses
// (16, 8, 4, or 0 when clusters cannot be launched).
int af_cluster_max(int M);

// The judge of a warm-started frame: the final image entropies of img (the
// plain leg) and img_l (the learned leg), M*512 floats each; img_l is copied
// over img when its entropy is lower, and stat[2] (the autofocus statistics)
// records the choice, stat[1] the kept leg's entropy of the selected bins.
// part: kJudgeParts * 4 doubles of scratch.
constexpr int kJudgeParts = 256;   // CTAs per image of the entropy sums
constexpr int kJudgeCopy = 128;    // CTAs of the decision and copy
cudaError_t img_judge(float* img, const float* img_l, int n, double* part, int* stat, cudaStream_t st);

struct PostArgs {
    int M;
    int data_type;           // 1 IFDS, 2 STRETCH
    int mtrc;
    float2* cut;             // [M][512]
    float2* st;              // [M][512] scratch
    float2* st2;             // [M][512] scratch
    const float2* pre;       // [M][512] a^-k * ww[M-1+k]
    const float2* post;      // [M][512] ww[M-1+k]
    const float2* V;         // [512][L] FFT_L(1/ww)
    const float* hamM;       // [M]
    float* img;              // [M][512]
    const float2* tw;
    // MTRC at M >= 512 only: the per-pulse phase the imaging applies to the
    // cut (the CZT's load; a row transform commutes with a per-row factor),
    // or nullptr when the cut is already phased; rows_ready: st already
    // holds the rows' transform of this cut (the second leg of a frame).
    const float2* phase;
    int rows_ready;
};

cudaError_t hpc_coef(const double* vel, int M, double coef_over_fs2, int64_t* hq, cudaStream_t st);
cudaError_t hpc_apply(float2* x, const int64_t* hq, int M, int N, cudaStream_t st);
cudaError_t ifds_pre(float2* x, int M, int N, const float2* tw, cudaStream_t st);
// getHRRP (common.cu:541-580) of `rows` rows of n cells; ham = hamming(n).
cudaError_t hrrp(const float2* x, float2* out, int rows, int n, const float* ham, int ifds, const float2* tw,
                 cudaStream_t st);

// IFDS pulse compression (common.cu:583-604, 635-746), one CTA per pulse.
struct PCArgs {
    int pulses;
    int iq_len;              // complex samples per pulse
    int ad_stride;           // int16 per pulse (even, >= 2 * iq_len)
    int nfft;                // nextPow2(iq_len): 4096, 8192 or 16384
    int S;                   // (int)(Fs * Tp) reference samples
    float fc_f;              // (float)fc
    float c2;                // (float)((double)(PI_FLT * (float)B) / Tp)
    float tp_f;              // (float)Tp
    const int16_t* ad;       // [pulses][ad_stride], I and Q interleaved
    const double* vel;       // [pulses] m/s
    float2* spec;            // [pulses][nfft] scratch
    float2* out;             // [pulses][out_stride], 4096 cells each
    int out_stride;          // float2 per output pulse
    int* offsets;            // [pulses] cut offsets, or nullptr
    const float2* tw;        // twiddle table exp(-2 pi i k / kTwN)
};
int pc_nfft(int iq_len);
// int16 I/Q pairs -> complex64 (samples complex values; in 8-byte and out
// 16-byte aligned).
cudaError_t iq16_to_c64(const int16_t* in, float* out, size_t samples, cudaStream_t st);
cudaError_t pulse_compress(const PCArgs& a, cudaStream_t st);
cudaError_t ra_run(const RAArgs& a, cudaStream_t st);
cudaError_t arp_from_y(const float2* y, int M, int N, float* tmp, unsigned* hmax, float* arp, cudaStream_t st);
cudaError_t center_cut(const float* arp, const float2* y, int M, int N, int* dec, float2* cut, cudaStream_t st);
// Raises k_center's dynamic shared-memory limit to the kMaxN case on the
// calling thread's current device (the attribute is per device).
cudaError_t center_prepare_current_device();

// Records `msg` as the calling thread's last error (isar_get_last_error)
// and returns `code`.
int record_error(int code, const char* msg);
cudaError_t fe_run(const FEArgs& a, cudaStream_t st);
cudaError_t post_run(const PostArgs& a, cudaStream_t st);
cudaError_t fft_rows(float2* x, int rows, int n, int inverse, const float2* tw, cudaStream_t st);

}  // namespace isar
