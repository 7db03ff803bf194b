// C ABI of the GB300 ISAR imaging library: context (workspace + tables),
// the per-frame pipeline and the stage entry points.
//
// The pipeline follows ISAR_RD_Imaging_Main_Ku (isar_main.cu:3-227):
//   [IFDS pre-step] -> HPC (fused into the range-alignment loads) -> range
//   alignment -> HRRPCenter + cut -> fastEntropy -> [MTRC] -> post.
// All launches are stream-ordered on the context stream; the only host
// synchronisation of a frame is the final image copy of isar_image_host.
#include <cuda_runtime.h>

#include <cmath>
#include <complex>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <algorithm>
#include <vector>

#include "../../include/isar_gb300.h"
#include "isar_common.cuh"
#include "isar_kernels.h"
#include "isar_synth.h"
#include "nn.h"

using isar::kRangeCut;

// defined with the network's C ABI (nn_api.cu)
const isar::nn::Weights* isar_wsnet_weights(const isar_wsnet* n);

namespace {

thread_local std::string g_last_error;

int fail(int code, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

#define CU(call)                                                                                   \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            return fail(ISAR_ECUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                        __LINE__);                                                                 \
    } while (0)

bool is_pow2(long v) { return v > 0 && (v & (v - 1)) == 0; }

// ---- host-side tables (float parameters rounded as the reference) --------
constexpr float kPiF = 3.14159265358979f;

// genHammingVec (common.cu:260-266)
void hamming_f32(float* w, int len)
{
    for (int i = 0; i < len; ++i) {
        float arg = 2 * kPiF * (float)i / (float)(len - 1);
        w[i] = 0.54f - 0.46f * (float)std::cos((double)arg);
    }
}

using cd = std::complex<double>;

void fft_host(std::vector<cd>& x, bool inverse)
{
    const int n = (int)x.size();
    for (int i = 1, j = 0; i < n; ++i) {
        int bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) std::swap(x[i], x[j]);
    }
    const double sgn = inverse ? 1.0 : -1.0;
    for (int len = 2; len <= n; len <<= 1) {
        const int half = len >> 1;
        for (int k = 0; k < half; ++k) {
            const double ang = sgn * 2.0 * M_PI * (double)k / (double)len;
            const cd w(std::cos(ang), std::sin(ang));
            for (int s = 0; s < n; s += len) {
                cd t = x[s + k + half] * w;
                x[s + k + half] = x[s + k] - t;
                x[s + k] = x[s + k] + t;
            }
        }
    }
}

// exp(y * log(z)) for the float-valued complex z, in double (thrust::pow's
// formula, mtrc.cu:87,102).
cd cpow_f32base(float re, float im, double y)
{
    const double lr = 0.5 * std::log1p(((double)re - 1.0) * ((double)re + 1.0) + (double)im * (double)im);
    const double th = std::atan2((double)im, (double)re);
    const double mag = std::exp(y * lr);
    return cd(mag * std::cos(y * th), mag * std::sin(y * th));
}

int next_pow2(int n)   // common.cu:521-529
{
    int r = 1;
    while (n >> 1) {
        r <<= 1;
        n >>= 1;
    }
    return r << 1;
}

struct FrameKey {
    const void* x;
    const void* vel;
    const void* img;
    int flags;
    bool operator==(const FrameKey& o) const { return x == o.x && vel == o.vel && img == o.img && flags == o.flags; }
};

struct CachedGraph {
    FrameKey key;
    cudaGraphExec_t exec;
    long long kernels;   // kernels per replay (for the launch counter)
    unsigned long long tick;
};

}  // namespace

int isar::record_error(int code, const char* msg) { return fail(code, "%s", msg); }

struct isar_ctx {
    isar_radar r{};
    int M = 0, N = 0, dev = 0;
    cudaStream_t st = nullptr;
    bool own_stream = false;
    bool imaged = false;
    // frame data: d_in = host frame staging, d_x = range profiles
    float2* d_in = nullptr;
    float2* d_x = nullptr;
    double* d_vel = nullptr;
    float* d_img = nullptr;
    // range alignment
    float* d_win = nullptr;
    float* d_win_hrrp = nullptr;   // d_win * hamming (if_hrrp on STRETCH data)
    float* d_ham = nullptr;        // hamming(N) (getHRRP)
    int64_t* d_hq = nullptr;
    double* d_S = nullptr;
    int64_t* d_SQ = nullptr;
    float* d_shifts = nullptr;
    float* d_env_a = nullptr;
    float* d_env_b = nullptr;
    float* d_part = nullptr;
    float* d_arp = nullptr;
    unsigned* d_hmax = nullptr;
    int* d_dec = nullptr;
    // cut and autofocus
    float2* d_cut = nullptr;
    float* d_cmax_part = nullptr;
    float2* d_dsum = nullptr;
    float2* d_phase = nullptr;
    int* d_fdec = nullptr;
    double* d_E = nullptr;
    double* d_H = nullptr;
    int* d_bins = nullptr;
    float2* d_sig_part = nullptr;
    float2* d_gcol = nullptr;
    // IFDS pulse compression: spectra of the pulses in flight (grown on demand)
    float2* d_pc_spec = nullptr;
    size_t pc_spec_len = 0;
    unsigned* d_bar = nullptr;     // [0] autofocus grid-barrier counter, [1] its timeout flag,
                                   // [2] range-alignment row-copy timeout flag
    // MTRC / post
    float2* d_st = nullptr;
    float2* d_st2 = nullptr;
    float2* d_pre = nullptr;
    float2* d_post = nullptr;
    float2* d_V = nullptr;
    float* d_hamM = nullptr;
    float2* d_tw = nullptr;
    std::vector<void*> allocs;
    double hpc_coef_over_fs2 = 0.0;
    bool ra_given = false;         // range alignment uses injected shifts (test hook)
    isar::BarrierTest bar_test;    // autofocus grid-barrier poll limit (test hook)
    // tuning (isar_set_tuning / the autotuner); defaults as the reference
    int ra_rows_each_level = 0;    // 0: spectral envelope merge
    int ra_pair_min = 128;
    int ra_rpc = 4;
    int ra_rpc_final = 4;
    int af_cluster = 0;
    float af_tol = 0.0f;
    int af_iters = isar::kEntropyIters;
    // cached CUDA graphs of whole frames
    bool use_graphs = true;
    std::vector<CachedGraph> graphs;
    unsigned long long graph_tick = 0;
    // learned warm start: the attached network and this context's
    // inference buffers (M rows)
    const isar::nn::Weights* ws_w = nullptr;
    isar::nn::Acts ws_a;
    float* d_ws_psi = nullptr;
    float2* d_ws_phase = nullptr;
    float2* d_cut2 = nullptr;      // the learned leg's cut, image and judge scratch
    float* d_img2 = nullptr;
    double* d_judge = nullptr;
    int* d_ws_err = nullptr;
    bool ws_alloc = false;
};

namespace {

template <class T>
int dalloc(isar_ctx* c, T** p, size_t count)
{
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, count * sizeof(T) + 256);
    if (e != cudaSuccess) return fail(ISAR_ENOMEM, "cudaMalloc(%zu) failed: %s", count * sizeof(T), cudaGetErrorString(e));
    c->allocs.push_back(q);
    *p = reinterpret_cast<T*>(q);
    return ISAR_OK;
}

void free_all(isar_ctx* c)
{
    for (void* p : c->allocs) cudaFree(p);
    c->allocs.clear();
}

#define TRY(x)                 \
    do {                       \
        int rc_ = (x);         \
        if (rc_ != ISAR_OK) {  \
            return rc_;        \
        }                      \
    } while (0)

int build_tables(isar_ctx* c)
{
    const int M = c->M, N = c->N, C = kRangeCut;
    // twiddles exp(-2 pi i k / kTwN)
    std::vector<float2> tw(isar::kTwN);
    for (int k = 0; k < isar::kTwN; ++k) {
        const double a = -2.0 * M_PI * (double)k / (double)isar::kTwN;
        tw[k] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
    CU(cudaMemcpyAsync(c->d_tw, tw.data(), tw.size() * sizeof(float2), cudaMemcpyHostToDevice, c->st));
    // range-alignment window: hamming(n) * cos(pi * n) (range_alignment.cu:195-201)
    std::vector<float> ham(N), win(N);
    hamming_f32(ham.data(), N);
    for (int n = 0; n < N; ++n) win[n] = ham[n] * (float)std::cos((double)(kPiF * (float)n));
    CU(cudaMemcpyAsync(c->d_win, win.data(), N * sizeof(float), cudaMemcpyHostToDevice, c->st));
    CU(cudaMemcpyAsync(c->d_ham, ham.data(), N * sizeof(float), cudaMemcpyHostToDevice, c->st));
    // getHRRP windows the STRETCH echoes in place before range alignment
    // (common.cu:565): x * hamming, then x * (hamming * cos(pi n))
    std::vector<float> win_h(N);
    for (int n = 0; n < N; ++n) win_h[n] = ham[n] * win[n];
    CU(cudaMemcpyAsync(c->d_win_hrrp, win_h.data(), N * sizeof(float), cudaMemcpyHostToDevice, c->st));
    std::vector<float> hm(M);
    hamming_f32(hm.data(), M);
    CU(cudaMemcpyAsync(c->d_hamM, hm.data(), M * sizeof(float), cudaMemcpyHostToDevice, c->st));
    // HPC coefficient / Fs^2 (high_speed_compensation.cu:17-18)
    const double chirp = (double)c->r.band_width / c->r.Tp;
    const double coef = -4.0 * isar::kPiD * chirp / isar::kLightSpeed;
    c->hpc_coef_over_fs2 = coef / ((double)c->r.Fs * (double)c->r.Fs);
    // CZT tables (mtrc.cu:10-12,47, getWandA :175-192, genWW :79-93, gety :96-109)
    const float chirp_rate = (float)c->r.band_width / (float)c->r.Tp;
    const float posa = chirp_rate * (float)c->r.Tp / ((float)c->r.fc * ((float)C - 1.0f));
    const float constant = chirp_rate * (float)c->r.Tp / (float)(2 * c->r.fc);
    const int L = next_pow2(2 * M - 1);
    const int wwl = 2 * M - 1;
    std::vector<float2> pre((size_t)M * C), post((size_t)M * C), V((size_t)C * L);
    std::vector<cd> ww(wwl), v(L);
    for (int cc = 0; cc < C; ++cc) {
        const float base = std::fmaf(posa, (float)cc, 1 - constant);
        const float tw_ = -2 * kPiF * base / (float)M;
        const float ta = -1 * kPiF * base;
        const float wre = (float)std::cos((double)tw_), wim = (float)std::sin((double)tw_);
        const float are = (float)std::cos((double)ta), aim = (float)std::sin((double)ta);
        for (int k = 0; k < wwl; ++k) {
            const int kk = k - (M - 1);
            const float kk2 = (float)(kk * kk) / 2.0f;
            ww[k] = cpow_f32base(wre, wim, (double)kk2);
        }
        for (int k = 0; k < M; ++k) {
            const cd p = cpow_f32base(are, aim, -(double)k) * ww[M - 1 + k];
            pre[(size_t)k * C + cc] = make_float2((float)p.real(), (float)p.imag());
            post[(size_t)k * C + cc] = make_float2((float)ww[M - 1 + k].real(), (float)ww[M - 1 + k].imag());
        }
        for (int k = 0; k < L; ++k) v[k] = (k < wwl) ? 1.0 / ww[k] : cd(0.0, 0.0);
        fft_host(v, false);
        for (int k = 0; k < L; ++k) V[(size_t)cc * L + k] = make_float2((float)v[k].real(), (float)v[k].imag());
    }
    CU(cudaMemcpyAsync(c->d_pre, pre.data(), pre.size() * sizeof(float2), cudaMemcpyHostToDevice, c->st));
    CU(cudaMemcpyAsync(c->d_post, post.data(), post.size() * sizeof(float2), cudaMemcpyHostToDevice, c->st));
    CU(cudaMemcpyAsync(c->d_V, V.data(), V.size() * sizeof(float2), cudaMemcpyHostToDevice, c->st));
    CU(cudaStreamSynchronize(c->st));
    return ISAR_OK;
}

int create_impl(isar_ctx* c)
{
    const int M = c->M, N = c->N, C = kRangeCut;
    const size_t MN = (size_t)M * N;
    TRY(dalloc(c, &c->d_in, MN));
    TRY(dalloc(c, &c->d_x, MN));
    TRY(dalloc(c, &c->d_vel, M));
    TRY(dalloc(c, &c->d_img, (size_t)M * C));
    TRY(dalloc(c, &c->d_win, N));
    TRY(dalloc(c, &c->d_win_hrrp, N));
    TRY(dalloc(c, &c->d_ham, N));
    TRY(dalloc(c, &c->d_hq, M));
    TRY(dalloc(c, &c->d_S, M));
    TRY(dalloc(c, &c->d_SQ, M));
    TRY(dalloc(c, &c->d_shifts, M));
    // env_a holds M/2 merged spectra (N complex each) or, in its two halves,
    // the ping and pong envelopes of the carried-envelope path
    TRY(dalloc(c, &c->d_env_a, (size_t)M * N));
    c->d_env_b = c->d_env_a + (size_t)(M / 2) * N;
    TRY(dalloc(c, &c->d_part, (size_t)std::max(M / 2, 256) * N));
    TRY(dalloc(c, &c->d_arp, N));
    TRY(dalloc(c, &c->d_hmax, 4));
    TRY(dalloc(c, &c->d_dec, 16));
    TRY(dalloc(c, &c->d_cut, (size_t)M * C));
    TRY(dalloc(c, &c->d_cmax_part, (size_t)32 * C));
    TRY(dalloc(c, &c->d_dsum, M));
    TRY(dalloc(c, &c->d_phase, M));
    TRY(dalloc(c, &c->d_fdec, 16));
    TRY(dalloc(c, &c->d_E, C));
    TRY(dalloc(c, &c->d_H, C));
    TRY(dalloc(c, &c->d_bins, C));
    TRY(dalloc(c, &c->d_sig_part, (size_t)128 * M));
    TRY(dalloc(c, &c->d_gcol, (size_t)M * C));
    TRY(dalloc(c, &c->d_bar, 4));
    CU(cudaMemsetAsync(c->d_bar, 0, 4 * sizeof(unsigned), c->st));
    TRY(dalloc(c, &c->d_st, (size_t)M * C));
    TRY(dalloc(c, &c->d_st2, (size_t)M * C));
    TRY(dalloc(c, &c->d_pre, (size_t)M * C));
    TRY(dalloc(c, &c->d_post, (size_t)M * C));
    TRY(dalloc(c, &c->d_V, (size_t)C * 2 * M));
    TRY(dalloc(c, &c->d_hamM, M));
    TRY(dalloc(c, &c->d_tw, isar::kTwN));
    CU(cudaMemsetAsync(c->d_dec, 0, 16 * sizeof(int), c->st));
    CU(cudaMemsetAsync(c->d_fdec, 0, 16 * sizeof(int), c->st));
    return build_tables(c);
}

isar::RAArgs ra_args(isar_ctx* c, const float2* x, float2* y, bool hpc, bool hrrp)
{
    isar::RAArgs a{};
    a.M = c->M;
    a.N = c->N;
    a.x = x;
    a.y = y;
    a.win = hrrp ? c->d_win_hrrp : c->d_win;
    a.hq = hpc ? c->d_hq : nullptr;
    a.S = c->d_S;
    a.SQ = c->d_SQ;
    a.shifts = c->d_shifts;
    a.env_a = c->d_env_a;
    a.env_b = c->d_env_b;
    a.part = c->d_part;
    a.arp = c->d_arp;
    a.hmax = c->d_hmax;
    a.tw = c->d_tw;
    a.rows_each_level = c->ra_rows_each_level;
    a.pair_min = c->ra_pair_min;
    a.rpc = c->ra_rpc;
    a.rpc_final = c->ra_rpc_final;
    a.given_shifts = c->ra_given ? 1 : 0;
    a.err = c->d_bar + 2;
    return a;
}

isar::FEArgs fe_args(isar_ctx* c, float2* cut, int iters)
{
    isar::FEArgs a{};
    a.M = c->M;
    a.iters = iters;
    a.cut = cut;
    a.cmax_part = c->d_cmax_part;
    a.dsum = c->d_dsum;
    a.phase = c->d_phase;
    a.fdec = c->d_fdec;
    a.E = c->d_E;
    a.H = c->d_H;
    a.bins = c->d_bins;
    a.sig_part = c->d_sig_part;
    a.gcol = c->d_gcol;
    a.bar = c->d_bar;
    a.bar_test = c->bar_test;
    a.tw = c->d_tw;
    a.af_cluster = c->af_cluster;
    a.tol = c->af_tol;
    a.af_stat = c->d_fdec + 4;
    if (c->ws_w) {
        a.ws_w = c->ws_w;
        a.ws_a = &c->ws_a;
        a.ws_psi = c->d_ws_psi;
        a.ws_phase = c->d_ws_phase;
        a.ws_err = c->d_ws_err;
        a.cut2 = c->d_cut2;
    }
    return a;
}

isar::PostArgs post_args(isar_ctx* c, float2* cut, int flags, float* img)
{
    isar::PostArgs a{};
    a.M = c->M;
    a.data_type = c->r.data_type;
    a.mtrc = (flags & ISAR_FLAG_MTRC) ? 1 : 0;
    a.cut = cut;
    a.st = c->d_st;
    a.st2 = c->d_st2;
    a.pre = c->d_pre;
    a.post = c->d_post;
    a.V = c->d_V;
    a.hamM = c->d_hamM;
    a.img = img;
    a.tw = c->d_tw;
    return a;
}

int run_range_align(isar_ctx* c, const float2* x, float2* y, const double* d_vel, int flags)
{
    // rows are staged into shared memory by bulk copies (16-byte granules)
    if ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(y)) & 15)
        return fail(ISAR_EINVAL, "echo and range-profile buffers must be 16-byte aligned");
    const bool hpc = (flags & ISAR_FLAG_HPC) && c->r.data_type == ISAR_DATA_STRETCH;
    if (hpc) {
        if (!d_vel) return fail(ISAR_EINVAL, "ISAR_FLAG_HPC needs the pulse velocities");
        CU(isar::hpc_coef(d_vel, c->M, c->hpc_coef_over_fs2, c->d_hq, c->st));
    }
    const bool hrrp = (flags & ISAR_FLAG_HRRP) && c->r.data_type == ISAR_DATA_STRETCH;
    isar::RAArgs a = ra_args(c, x, y, hpc, hrrp);
    if (flags & ISAR_FLAG_IQ16) {
        // int16 samples: half the size of the profiles, so never in place
        if (reinterpret_cast<const void*>(x) == reinterpret_cast<const void*>(y))
            return fail(ISAR_EINVAL, "ISAR_FLAG_IQ16 needs separate echo and profile buffers");
        a.x_iq16 = 1;
    }
    CU(isar::ra_run(a, c->st));
    return ISAR_OK;
}

// x is read only, except for IFDS data whose pre-step works in place on a
// copy in the context (d_in).
int run_frame_eager(isar_ctx* c, const float2* x, const double* d_vel, int flags, float* d_img)
{
    if (c->r.data_type == ISAR_DATA_IFDS) {
        if (flags & ISAR_FLAG_IQ16)
            CU(isar::iq16_to_c64(reinterpret_cast<const int16_t*>(x), reinterpret_cast<float*>(c->d_in),
                                 (size_t)c->M * c->N, c->st));
        else if (x != c->d_in)
            CU(cudaMemcpyAsync(c->d_in, x, (size_t)c->M * c->N * sizeof(float2), cudaMemcpyDeviceToDevice, c->st));
        CU(isar::ifds_pre(c->d_in, c->M, c->N, c->d_tw, c->st));
        x = c->d_in;
        flags &= ~ISAR_FLAG_IQ16;
    }
    TRY(run_range_align(c, x, c->d_x, d_vel, flags));
    CU(isar::center_cut(c->d_arp, c->d_x, c->M, c->N, c->d_dec, c->d_cut, c->st));
    // With MTRC at 512 pulses or more the imaging applies the autofocus
    // phase itself (in the CZT's load), so the cut stays unphased and the
    // rows' transform of the MTRC is shared by both legs of a warm start.
    const bool fold = (flags & ISAR_FLAG_MTRC) && c->M >= 512;
    isar::FEArgs fa = fe_args(c, c->d_cut, c->af_iters);
    fa.defer_apply = fold ? 1 : 0;
    CU(isar::fe_run(fa, c->st));
    isar::PostArgs pa = post_args(c, c->d_cut, flags, d_img);
    if (fold) pa.phase = c->d_phase;
    CU(isar::post_run(pa, c->st));
    if (c->ws_w && c->af_iters > 0) {
        // warm start: image the learned leg too; the judge keeps the lower
        // final image entropy in d_img
        isar::PostArgs pl = post_args(c, fold ? c->d_cut : c->d_cut2, flags, c->d_img2);
        if (fold) {
            pl.phase = c->d_ws_phase;
            pl.rows_ready = 1;
        }
        CU(isar::post_run(pl, c->st));
        CU(isar::img_judge(d_img, c->d_img2, c->M * kRangeCut, c->d_judge, c->d_fdec + 4, c->st));
    }
    return ISAR_OK;
}

// One frame.  The first frame of a context runs eagerly (it also sets the
// kernels' attributes); later frames replay a CUDA graph of the whole chain,
// captured once per (input, velocity, image, flags) and cached (LRU of 8).
int run_frame(isar_ctx* c, const float2* x, const double* d_vel, int flags, float* d_img)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    CU(cudaStreamIsCapturing(c->st, &cs));
    if (!c->imaged || cs != cudaStreamCaptureStatusNone || !c->use_graphs) {
        TRY(run_frame_eager(c, x, d_vel, flags, d_img));
        c->imaged = true;
        return ISAR_OK;
    }
    const FrameKey key{x, d_vel, d_img, flags};
    ++c->graph_tick;
    for (auto& g : c->graphs)
        if (g.key == key) {
            g.tick = c->graph_tick;
            CU(cudaGraphLaunch(g.exec, c->st));
            isar::launch_counter() += g.kernels;
            return ISAR_OK;
        }
    const long long n0 = isar::launch_counter().load();
    CU(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeRelaxed));
    int rc = run_frame_eager(c, x, d_vel, flags, d_img);
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(c->st, &graph);
    if (rc != ISAR_OK) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    if (e != cudaSuccess) return fail(ISAR_ECUDA, "graph capture: %s", cudaGetErrorString(e));
    CachedGraph g{key, nullptr, isar::launch_counter().load() - n0, c->graph_tick};
    isar::launch_counter() = n0;
    e = cudaGraphInstantiate(&g.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return fail(ISAR_ECUDA, "graph instantiate: %s", cudaGetErrorString(e));
    if (c->graphs.size() >= 8) {
        auto lru = std::min_element(c->graphs.begin(), c->graphs.end(),
                                    [](const CachedGraph& a, const CachedGraph& b) { return a.tick < b.tick; });
        cudaGraphExecDestroy(lru->exec);
        c->graphs.erase(lru);
    }
    c->graphs.push_back(g);
    CU(cudaGraphLaunch(g.exec, c->st));
    isar::launch_counter() += g.kernels;
    return ISAR_OK;
}

int check_ctx(isar_ctx* c)
{
    if (!c) return fail(ISAR_EINVAL, "null context");
    CU(cudaSetDevice(c->dev));
    return ISAR_OK;
}

// Waits for the context stream and reports device-side failures: the
// autofocus kernel's grid barrier and the range-alignment row copies set a
// flag instead of waiting forever.
int sync_status(isar_ctx* c)
{
    CU(cudaStreamSynchronize(c->st));
    unsigned flag[3] = {0, 0, 0};
    CU(cudaMemcpy(flag, c->d_bar, sizeof(flag), cudaMemcpyDeviceToHost));
    if (flag[1] || flag[2]) {
        CU(cudaMemsetAsync(c->d_bar, 0, 3 * sizeof(unsigned), c->st));
        CU(cudaStreamSynchronize(c->st));
        return fail(ISAR_ECUDA, flag[1] ? "autofocus grid barrier timed out (image of this frame is invalid)"
                                        : "range-alignment row copy timed out (image of this frame is invalid)");
    }
    return ISAR_OK;
}

}  // namespace

extern "C" {

ISAR_API int isar_get_last_error(char* buf, size_t len)
{
    if (buf && len) {
        std::strncpy(buf, g_last_error.c_str(), len - 1);
        buf[len - 1] = 0;
    }
    return (int)g_last_error.size();
}

ISAR_API const char* isar_version(void) { return "isar_gb300 0.1 (sm_103a)"; }

ISAR_API long long isar_launch_count(void) { return isar::launch_counter().load(); }

ISAR_API int isar_create(isar_ctx** out, const isar_radar* radar, int device, void* stream)
{
    if (!out || !radar) return fail(ISAR_EINVAL, "null argument");
    *out = nullptr;
    const int M = radar->echo_num, N = radar->range_num;
    // guards of imagingMemInit (isar_imaging_export.cpp:144-155), plus the
    // power-of-two sizes the kernels are built for
    if (M > isar::kMaxM) return fail(ISAR_EINVAL, "echo_num %d > %d", M, isar::kMaxM);
    if (N < kRangeCut) return fail(ISAR_EINVAL, "range_num %d < range_num_cut %d", N, kRangeCut);
    if (N < M) return fail(ISAR_EINVAL, "range_num %d < echo_num %d", N, M);
    if (!is_pow2(M) || M < 128) return fail(ISAR_EINVAL, "echo_num %d: a power of two >= 128 is required", M);
    if (!is_pow2(N) || N > isar::kMaxN)
        return fail(ISAR_EINVAL, "range_num %d: a power of two <= %d is required", N, isar::kMaxN);
    if (radar->data_type != ISAR_DATA_STRETCH && radar->data_type != ISAR_DATA_IFDS)
        return fail(ISAR_EINVAL, "data_type %d", radar->data_type);
    if (!(radar->Tp > 0) || radar->Fs <= 0 || radar->fc <= 0 || radar->band_width <= 0)
        return fail(ISAR_EINVAL, "radar parameters must be positive");
    int ndev = 0;
    CU(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) return fail(ISAR_EINVAL, "device %d of %d", device, ndev);
    CU(cudaSetDevice(device));
    isar_ctx* c = new isar_ctx();
    c->r = *radar;
    c->M = M;
    c->N = N;
    c->dev = device;
    if (stream) {
        c->st = (cudaStream_t)stream;
    } else {
        cudaError_t e = cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            delete c;
            return fail(ISAR_ECUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
        }
        c->own_stream = true;
    }
    int rc = create_impl(c);
    if (rc != ISAR_OK) {
        std::string msg = g_last_error;
        isar_destroy(c);
        g_last_error = msg;
        return rc;
    }
    // Default autofocus engine: the fastest for one frame of M pulses,
    // measured on a GB300 with the reference's 120 iterations (U = 64..128
    // selected bins): clusters of 4 / 8 CTAs at 128 / 256 pulses, the
    // cooperative grid at 512, clusters of 16 at 1024; the cooperative grid
    // where the device cannot launch that cluster.  Every engine computes
    // the reference's iteration (the same parity bar).
    const int pref = M == 128 ? 4 : M == 256 ? 8 : M == 1024 ? 16 : 0;
    c->af_cluster = (pref > 0 && isar::af_cluster_max(M) >= pref) ? pref : 0;
    *out = c;
    return ISAR_OK;
}

ISAR_API int isar_destroy(isar_ctx* c)
{
    if (!c) return ISAR_OK;
    cudaSetDevice(c->dev);
    if (c->st) cudaStreamSynchronize(c->st);
    for (auto& g : c->graphs) cudaGraphExecDestroy(g.exec);
    c->graphs.clear();
    free_all(c);
    if (c->own_stream && c->st) cudaStreamDestroy(c->st);
    delete c;
    return ISAR_OK;
}

ISAR_API void* isar_stream(isar_ctx* c) { return c ? (void*)c->st : nullptr; }

ISAR_API int isar_image_host(isar_ctx* c, const float* echo, const double* velocity, int flags, float* img)
{
    TRY(check_ctx(c));
    if (!echo || !img) return fail(ISAR_EINVAL, "null echo/img");
    if (flags & ISAR_FLAG_IQ16) return fail(ISAR_EINVAL, "ISAR_FLAG_IQ16 applies to device buffers only");
    const size_t MN = (size_t)c->M * c->N;
    CU(cudaMemcpyAsync(c->d_in, echo, MN * sizeof(float2), cudaMemcpyHostToDevice, c->st));
    const double* dv = nullptr;
    if (velocity) {
        CU(cudaMemcpyAsync(c->d_vel, velocity, c->M * sizeof(double), cudaMemcpyHostToDevice, c->st));
        dv = c->d_vel;
    }
    TRY(run_frame(c, c->d_in, dv, flags, c->d_img));
    CU(cudaMemcpyAsync(img, c->d_img, (size_t)c->M * kRangeCut * sizeof(float), cudaMemcpyDeviceToHost, c->st));
    return sync_status(c);
}

ISAR_API int isar_synchronize(isar_ctx* c)
{
    TRY(check_ctx(c));
    return sync_status(c);
}

ISAR_API int isar_set_ra_shifts(isar_ctx* c, const float* shifts)
{
    TRY(check_ctx(c));
    CU(cudaStreamSynchronize(c->st));
    if (shifts) CU(cudaMemcpy(c->d_shifts, shifts, (c->M - 1) * sizeof(float), cudaMemcpyHostToDevice));
    c->ra_given = shifts != nullptr;
    for (auto& g : c->graphs) cudaGraphExecDestroy(g.exec);   // graphs bake the flag in
    c->graphs.clear();
    return ISAR_OK;
}

ISAR_API int isar_test_barrier_timeout(isar_ctx* c, unsigned polls, int never_complete)
{
    TRY(check_ctx(c));
    if (polls == 0 && never_complete) return fail(ISAR_EINVAL, "a barrier that never completes needs a poll limit");
    CU(cudaStreamSynchronize(c->st));
    c->bar_test.limit = polls ? polls : isar::kSpinLimit;
    c->bar_test.extra = never_complete ? 1u : 0u;
    for (auto& g : c->graphs) cudaGraphExecDestroy(g.exec);   // graphs bake the kernel arguments in
    c->graphs.clear();
    return ISAR_OK;
}

ISAR_API int isar_image_device(isar_ctx* c, const float* d_echo, const double* d_velocity, int flags, float* d_img)
{
    TRY(check_ctx(c));
    if (!d_echo || !d_img) return fail(ISAR_EINVAL, "null echo/img");
    return run_frame(c, reinterpret_cast<const float2*>(d_echo), d_velocity, flags, d_img);
}

ISAR_API int isar_get_profiles(isar_ctx* c, const float** d_profiles)
{
    TRY(check_ctx(c));
    if (!d_profiles) return fail(ISAR_EINVAL, "null argument");
    *d_profiles = reinterpret_cast<const float*>(c->d_x);
    return ISAR_OK;
}

ISAR_API int isar_synth_device(const isar_synth_params* p, float* d_out, double* d_velocity, double* h_velocity,
                               void* stream)
{
    if (!p || !d_out) return fail(ISAR_EINVAL, "null argument");
    if (p->M <= 0 || p->N <= 0 || p->n_scat < 0 || p->n_scat > 4096 || !(p->Fs > 0) || !(p->B > 0))
        return fail(ISAR_EINVAL, "bad synthetic frame parameters");
    isar::SynthParams q{};
    q.M = p->M;
    q.N = p->N;
    q.fc = p->fc;
    q.B = p->B;
    q.prf = p->prf;
    q.Fs = p->Fs;
    q.n_scat = p->n_scat;
    q.patch_x = p->patch_x;
    q.patch_y = p->patch_y;
    q.omega = p->omega;
    q.r0_cells = p->r0_cells;
    q.drift_sigma = p->drift_sigma;
    q.phase_uniform = p->phase_uniform;
    q.phase_quad = p->phase_quad;
    q.v0 = p->v0;
    q.accel = p->accel;
    q.snr_db = p->snr_db;
    q.rms_counts = p->rms_counts;
    q.seed = p->seed;
    q.phase_poly_order = p->phase_poly_order;
    q.phase_poly_sigma = p->phase_poly_sigma;
    q.h_phase_err = p->h_phase_err;
    int64_t* scratch = nullptr;
    CU(cudaMalloc(&scratch, (size_t)p->M * (p->n_scat > 0 ? p->n_scat : 1) * 4 * sizeof(int64_t)));
    cudaError_t e = isar::synth_frame(q, reinterpret_cast<float2*>(d_out), d_velocity, h_velocity, scratch,
                                      (cudaStream_t)stream);
    cudaFree(scratch);
    if (e != cudaSuccess) return fail(ISAR_ECUDA, "synthetic frame: %s", cudaGetErrorString(e));
    return ISAR_OK;
}

ISAR_API int isar_get_trace(isar_ctx* c, isar_trace* t)
{
    TRY(check_ctx(c));
    if (!t) return fail(ISAR_EINVAL, "null trace");
    int dec[16], fdec[16];
    CU(cudaMemcpyAsync(dec, c->d_dec, sizeof(dec), cudaMemcpyDeviceToHost, c->st));
    CU(cudaMemcpyAsync(fdec, c->d_fdec, sizeof(fdec), cudaMemcpyDeviceToHost, c->st));
    CU(cudaMemcpyAsync(t->bins, c->d_bins, sizeof(t->bins), cudaMemcpyDeviceToHost, c->st));
    if (t->ra_shift)
        CU(cudaMemcpyAsync(t->ra_shift, c->d_shifts, (c->M - 1) * sizeof(float), cudaMemcpyDeviceToHost, c->st));
    if (t->phase)
        CU(cudaMemcpyAsync(t->phase, c->d_phase, c->M * sizeof(float2), cudaMemcpyDeviceToHost, c->st));
    TRY(sync_status(c));
    t->center_applied = dec[0];
    t->center_shift = dec[1];
    t->cut_offset = dec[2];
    t->center_idx1_len = dec[3];
    t->center_idx2_len = dec[4];
    std::memcpy(&t->center_threshold, &dec[5], sizeof(float));
    t->tgt_num = fdec[0];
    t->unit2_num = fdec[1];
    for (int i = t->unit2_num; i < 512; ++i) t->bins[i] = 0;
    if (c->af_cluster > 0) {
        t->af_iterations = fdec[4];
        std::memcpy(&t->af_entropy, &fdec[5], sizeof(float));
    } else {
        t->af_iterations = c->af_iters;
        t->af_entropy = NAN;
    }
    t->ws_used = c->ws_w ? fdec[6] : 0;
    if (c->ws_w) {
        std::memcpy(&t->af_entropy_final[0], &fdec[7], sizeof(float));
        std::memcpy(&t->af_entropy_final[1], &fdec[8], sizeof(float));
        t->af_iterations_leg[0] = fdec[9];
        t->af_iterations_leg[1] = fdec[10];
    } else {
        t->af_entropy_final[0] = t->af_entropy_final[1] = NAN;
        t->af_iterations_leg[0] = t->af_iterations_leg[1] = 0;
    }
    return ISAR_OK;
}

ISAR_API int isar_set_warmstart(isar_ctx* c, const isar_wsnet* net)
{
    TRY(check_ctx(c));
    if (net && c->af_cluster == 0)
        return fail(ISAR_EINVAL, "the learned warm start needs the cluster autofocus engine (isar_set_tuning)");
    CU(cudaStreamSynchronize(c->st));
    if (net && !c->ws_alloc) {
        const size_t M = c->M;
        c->ws_a.rows = c->M;
        for (int l = 0; l < isar::nn::kConv + 2; ++l) TRY(dalloc(c, &c->ws_a.act[l], M * isar::nn::kCh));
        TRY(dalloc(c, &c->ws_a.col, M * isar::nn::kColK));
        TRY(dalloc(c, &c->ws_a.out, M * isar::nn::kOutPad));
        TRY(dalloc(c, &c->d_ws_psi, M));
        TRY(dalloc(c, &c->d_ws_phase, M));
        TRY(dalloc(c, &c->d_ws_err, 1));
        TRY(dalloc(c, &c->d_cut2, M * kRangeCut));
        TRY(dalloc(c, &c->d_img2, M * kRangeCut));
        TRY(dalloc(c, &c->d_judge, (size_t)isar::kJudgeParts * 4));
        CU(cudaMemsetAsync(c->d_ws_err, 0, sizeof(int), c->st));
        c->ws_alloc = true;
    }
    c->ws_w = net ? isar_wsnet_weights(net) : nullptr;
    for (auto& g : c->graphs) cudaGraphExecDestroy(g.exec);
    c->graphs.clear();
    return ISAR_OK;
}

ISAR_API int isar_frame_features(isar_ctx* c, const float* d_echo, const double* d_velocity, int flags, void* d_x0,
                                 float* d_psi)
{
    TRY(check_ctx(c));
    if (!d_echo || !d_x0 || !d_psi) return fail(ISAR_EINVAL, "null argument");
    const float2* x = reinterpret_cast<const float2*>(d_echo);
    if (c->r.data_type == ISAR_DATA_IFDS) {
        CU(cudaMemcpyAsync(c->d_in, x, (size_t)c->M * c->N * sizeof(float2), cudaMemcpyDeviceToDevice, c->st));
        CU(isar::ifds_pre(c->d_in, c->M, c->N, c->d_tw, c->st));
        x = c->d_in;
    }
    TRY(run_range_align(c, x, c->d_x, d_velocity, flags));
    CU(isar::center_cut(c->d_arp, c->d_x, c->M, c->N, c->d_dec, c->d_cut, c->st));
    isar::FEArgs a = fe_args(c, c->d_cut, 0);
    a.ws_w = nullptr;
    a.pre_only = 1;
    CU(isar::fe_run(a, c->st));
    CU(isar::nn::features(c->d_cut, c->d_E, c->d_dsum, c->M, static_cast<__nv_bfloat16*>(d_x0), d_psi, c->st));
    return ISAR_OK;
}

ISAR_API int isar_get_tuning(isar_ctx* c, isar_tuning* t)
{
    TRY(check_ctx(c));
    if (!t) return fail(ISAR_EINVAL, "null tuning");
    t->ra_rows_each_level = c->ra_rows_each_level;
    t->ra_pair_min = c->ra_pair_min;
    t->ra_rows_per_cta = c->ra_rpc;
    t->ra_rows_final = c->ra_rpc_final;
    t->af_cluster = c->af_cluster;
    t->af_tol = c->af_tol;
    t->af_iters = c->af_iters;
    t->af_cluster_max = isar::af_cluster_max(c->M);
    return ISAR_OK;
}

ISAR_API int isar_set_tuning(isar_ctx* c, const isar_tuning* t)
{
    TRY(check_ctx(c));
    if (!t) return fail(ISAR_EINVAL, "null tuning");
    if (t->ra_pair_min < 1 || !is_pow2(t->ra_rows_per_cta) || !is_pow2(t->ra_rows_final) || t->ra_rows_per_cta > 64 ||
        t->ra_rows_final > 64)
        return fail(ISAR_EINVAL, "range-alignment tuning out of range");
    if (t->ra_rows_each_level != 0 && t->ra_rows_each_level != 1)
        return fail(ISAR_EINVAL, "ra_rows_each_level must be 0 or 1");
    if (t->af_cluster != 0 && t->af_cluster != 4 && t->af_cluster != 8 && t->af_cluster != 16)
        return fail(ISAR_EINVAL, "af_cluster must be 0, 4, 8 or 16");
    if (t->af_cluster > isar::af_cluster_max(c->M))
        return fail(ISAR_EINVAL, "af_cluster %d exceeds what this device can launch (%d)", t->af_cluster,
                    isar::af_cluster_max(c->M));
    if (t->af_tol < 0.0f || !(t->af_tol < 1.0f)) return fail(ISAR_EINVAL, "af_tol must be in [0, 1)");
    if (t->af_tol > 0.0f && t->af_cluster == 0) return fail(ISAR_EINVAL, "af_tol needs the cluster engine");
    if (c->ws_w && t->af_cluster == 0) return fail(ISAR_EINVAL, "the attached warm start needs the cluster engine");
    if (t->af_iters < 0 || t->af_iters > 100000) return fail(ISAR_EINVAL, "af_iters out of range");
    CU(cudaStreamSynchronize(c->st));
    c->ra_rows_each_level = t->ra_rows_each_level;
    c->ra_pair_min = t->ra_pair_min;
    c->ra_rpc = t->ra_rows_per_cta;
    c->ra_rpc_final = t->ra_rows_final;
    c->af_cluster = t->af_cluster;
    c->af_tol = t->af_tol;
    c->af_iters = t->af_iters;
    for (auto& g : c->graphs) cudaGraphExecDestroy(g.exec);
    c->graphs.clear();
    return ISAR_OK;
}

ISAR_API int isar_stage_hpc(isar_ctx* c, float* d_x, const double* d_velocity)
{
    TRY(check_ctx(c));
    if (!d_x || !d_velocity) return fail(ISAR_EINVAL, "null argument");
    CU(isar::hpc_coef(d_velocity, c->M, c->hpc_coef_over_fs2, c->d_hq, c->st));
    CU(isar::hpc_apply(reinterpret_cast<float2*>(d_x), c->d_hq, c->M, c->N, c->st));
    return ISAR_OK;
}

ISAR_API int isar_stage_range_align(isar_ctx* c, float* d_x, const double* d_velocity, int flags)
{
    TRY(check_ctx(c));
    if (!d_x) return fail(ISAR_EINVAL, "null argument");
    float2* x = reinterpret_cast<float2*>(d_x);
    return run_range_align(c, x, x, d_velocity, flags);
}

ISAR_API int isar_stage_center_cut(isar_ctx* c, const float* d_y, float* d_cut)
{
    TRY(check_ctx(c));
    if (!d_y || !d_cut) return fail(ISAR_EINVAL, "null argument");
    const float2* y = reinterpret_cast<const float2*>(d_y);
    CU(isar::arp_from_y(y, c->M, c->N, c->d_part, c->d_hmax, c->d_arp, c->st));
    CU(isar::center_cut(c->d_arp, y, c->M, c->N, c->d_dec, reinterpret_cast<float2*>(d_cut), c->st));
    return ISAR_OK;
}

ISAR_API int isar_stage_fast_entropy(isar_ctx* c, float* d_cut, int iterations)
{
    TRY(check_ctx(c));
    if (!d_cut || iterations < 0) return fail(ISAR_EINVAL, "bad argument");
    // the stage alone runs the plain autofocus: a warm start is judged on
    // final images, which only the whole frame produces
    isar::FEArgs a = fe_args(c, reinterpret_cast<float2*>(d_cut), iterations);
    a.ws_w = nullptr;
    CU(isar::fe_run(a, c->st));
    return ISAR_OK;
}

ISAR_API int isar_stage_post(isar_ctx* c, float* d_cut, int flags, float* d_img)
{
    TRY(check_ctx(c));
    if (!d_cut || !d_img) return fail(ISAR_EINVAL, "null argument");
    CU(isar::post_run(post_args(c, reinterpret_cast<float2*>(d_cut), flags, d_img), c->st));
    return ISAR_OK;
}

ISAR_API int isar_iq16_to_c64(const int16_t* d_iq, float* d_echo, size_t samples, void* stream)
{
    if ((!d_iq || !d_echo) && samples) return fail(ISAR_EINVAL, "null argument");
    if ((reinterpret_cast<uintptr_t>(d_iq) & 7) || (reinterpret_cast<uintptr_t>(d_echo) & 15))
        return fail(ISAR_EINVAL, "d_iq must be 8-byte and d_echo 16-byte aligned");
    CU(isar::iq16_to_c64(d_iq, d_echo, samples, static_cast<cudaStream_t>(stream)));
    return ISAR_OK;
}

ISAR_API int isar_stage_hrrp(isar_ctx* c, const float* d_x, float* d_hrrp)
{
    TRY(check_ctx(c));
    if (!d_x || !d_hrrp) return fail(ISAR_EINVAL, "null argument");
    CU(isar::hrrp(reinterpret_cast<const float2*>(d_x), reinterpret_cast<float2*>(d_hrrp), c->M, c->N, c->d_ham,
                  c->r.data_type == ISAR_DATA_IFDS ? 1 : 0, c->d_tw, c->st));
    return ISAR_OK;
}

ISAR_API int isar_pulse_compress(isar_ctx* c, const int16_t* d_ad, int iq_len, const double* d_velocity,
                                 int pulses, float* d_out, int* d_offsets)
{
    TRY(check_ctx(c));
    if (!d_ad || !d_velocity || !d_out || pulses < 0 || iq_len <= 0) return fail(ISAR_EINVAL, "bad argument");
    if ((reinterpret_cast<uintptr_t>(d_ad) & 3) || (reinterpret_cast<uintptr_t>(d_out) & 7))
        return fail(ISAR_EINVAL, "d_ad must be 4-byte and d_out 8-byte aligned");
    const int nfft = isar::pc_nfft(iq_len);
    const int S = (int)((double)c->r.Fs * c->r.Tp);
    if (nfft != 4096 && nfft != 8192 && nfft != 16384)
        return fail(ISAR_EINVAL, "nextPow2(iq_len) = %d: supported 4096, 8192, 16384", nfft);
    if (S < 2 || S > nfft) return fail(ISAR_EINVAL, "reference length Fs*Tp = %d outside [2, %d]", S, nfft);
    if (pulses == 0) return ISAR_OK;
    const size_t need = (size_t)pulses * nfft;
    if (need > c->pc_spec_len) {
        CU(cudaStreamSynchronize(c->st));
        if (c->d_pc_spec) {
            cudaFree(c->d_pc_spec);
            c->allocs.erase(std::find(c->allocs.begin(), c->allocs.end(), (void*)c->d_pc_spec));
            c->d_pc_spec = nullptr;
            c->pc_spec_len = 0;
        }
        TRY(dalloc(c, &c->d_pc_spec, need));
        c->pc_spec_len = need;
    }
    isar::PCArgs a{};
    a.pulses = pulses;
    a.iq_len = iq_len;
    a.ad_stride = 2 * iq_len;
    a.nfft = nfft;
    a.S = S;
    a.fc_f = (float)c->r.fc;
    a.c2 = (float)((double)(kPiF * (float)c->r.band_width) / c->r.Tp);   // genRefPulseCompression constant_2
    a.tp_f = (float)c->r.Tp;
    a.ad = d_ad;
    a.vel = d_velocity;
    a.spec = c->d_pc_spec;
    a.out = reinterpret_cast<float2*>(d_out);
    a.out_stride = isar::kRangeNumIfdsPc;
    a.offsets = d_offsets;
    a.tw = c->d_tw;
    CU(isar::pulse_compress(a, c->st));
    return ISAR_OK;
}

ISAR_API int isar_fft_rows(isar_ctx* c, float* d_x, int rows, int n, int inverse)
{
    TRY(check_ctx(c));
    if (!d_x || rows <= 0 || !is_pow2(n) || n < 512 || n > isar::kMaxN) return fail(ISAR_EINVAL, "bad fft size");
    CU(isar::fft_rows(reinterpret_cast<float2*>(d_x), rows, n, inverse, c->d_tw, c->st));
    return ISAR_OK;
}

}  // extern "C"
