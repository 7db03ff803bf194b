// On-GPU synthetic dechirped (STRETCH) echoes: rotating point-scatterer
// target, per-pulse range drift, phase error, radial velocity (the
// high-speed-compensation term) and complex white noise, quantised to int16
// ADC counts like the .wbd payload (common.cu:1085-1100).
//
// x[m,n] = sum_k a_k exp(-j (4 pi / c) (fc + K t_n) (R_k(m) - v_m t_n) + j phi_m)
//          + noise,  t_n = n / Fs,  K = B / Tp.
// Per (m, k) the phase in cycles is A0 + A1 n + A2 n^2; the three
// coefficients are reduced modulo one on the host in double and the sum is
// evaluated in 64-bit fixed point (exact modulo one cycle).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "isar_common.cuh"
#include "isar_kernels.h"
#include "isar_synth.h"

namespace isar {

__device__ __forceinline__ uint64_t mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// coef: [M][K][4] = {F0, F1, F2 (fixed point), amplitude bits}
__global__ void __launch_bounds__(256)
k_synth(const int64_t* __restrict__ coef, int K, int N, float scale, float nsig, uint64_t seed,
        float2* __restrict__ out)
{
    const int m = blockIdx.y;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    extern __shared__ int64_t sc[];
    for (int i = threadIdx.x; i < 4 * K; i += blockDim.x) sc[i] = coef[(size_t)m * K * 4 + i];
    __syncthreads();
    if (n >= N) return;
    const uint64_t nn = (uint64_t)n;
    const uint64_t n2 = nn * nn;
    float re = 0.0f, im = 0.0f;
    for (int k = 0; k < K; ++k) {
        const uint64_t ph = (uint64_t)sc[4 * k] + (uint64_t)sc[4 * k + 1] * nn + (uint64_t)sc[4 * k + 2] * n2;
        const float a = __int_as_float((int)sc[4 * k + 3]);
        const float2 c = cis_frac64(ph);
        re = fmaf(a, c.x, re);
        im = fmaf(a, c.y, im);
    }
    // Box-Muller noise from a counter hash
    const uint64_t h1 = mix64(seed ^ (((uint64_t)m << 32) | (uint64_t)n) ^ 0x9E3779B97F4A7C15ull);
    const uint64_t h2 = mix64(h1 + 0x632BE59BD9B4E019ull);
    const float u1 = ((float)(h1 >> 40) + 0.5f) * (1.0f / 16777216.0f);
    const float u2 = (float)(h2 >> 40) * (1.0f / 16777216.0f);
    const float r = sqrtf(-2.0f * logf(u1));
    float s, c;
    sincospif(2.0f * u2, &s, &c);
    re = (re + nsig * r * c) * scale;
    im = (im + nsig * r * s) * scale;
    re = fminf(fmaxf(rintf(re), -32768.0f), 32767.0f);
    im = fminf(fmaxf(rintf(im), -32768.0f), 32767.0f);
    out[(size_t)m * N + n] = make_float2(re, im);
}

namespace {

struct Rng {
    uint64_t s;
    uint64_t next()
    {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return ((double)(next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
    double gauss() { return std::sqrt(-2.0 * std::log(uniform())) * std::cos(2.0 * M_PI * uniform()); }
};

int64_t frac64(double v)
{
    v -= std::floor(v + 0.5);
    return (int64_t)std::llrint(std::ldexp(v, 64));
}

}  // namespace

cudaError_t synth_frame(const SynthParams& p, float2* d_out, double* d_vel, double* h_vel, int64_t* d_coef_scratch,
                        cudaStream_t st)
{
    const int M = p.M, N = p.N, K = p.n_scat;
    const double c = kLightSpeed;
    const double Tp = (double)N / p.Fs;
    const double Kr = p.B / Tp;
    const double cell = c / (2.0 * p.B);
    Rng rng{p.seed};
    std::vector<double> sx(K), sy(K), amp(K), ph0(K);
    double pw = 0.0;
    for (int k = 0; k < K; ++k) {
        sx[k] = (rng.uniform() - 0.5) * p.patch_x;
        sy[k] = (rng.uniform() - 0.5) * p.patch_y;
        amp[k] = std::sqrt(-2.0 * std::log(rng.uniform()));
        ph0[k] = rng.uniform();
        pw += amp[k] * amp[k];
    }
    std::vector<int64_t> coef((size_t)M * K * 4);
    std::vector<double> vel(M);
    // polynomial phase-error coefficients from their own stream, so that
    // frames without them are unchanged
    double poly[8] = {0.0};
    if (p.phase_poly_order >= 2) {
        Rng prng{p.seed ^ 0x5DEECE66Dull};
        for (int k = 2; k <= p.phase_poly_order && k < 8; ++k) poly[k] = p.phase_poly_sigma * prng.gauss();
    }
    double d = 0.0;
    for (int m = 0; m < M; ++m) {
        const double drift = d * cell;
        d += p.drift_sigma * rng.gauss();
        const double u = (double)(m - M / 2) / (double)(M / 2);
        double perr = p.phase_quad * u * u + p.phase_uniform * (2.0 * rng.uniform() - 1.0);
        double uk = u;
        for (int k = 2; k < 8; ++k) {
            uk *= u;
            perr += poly[k] * uk;
        }
        // the phase the autofocus has to remove: the injected error plus the
        // carrier phase of the translational range drift, -4 pi fc drift / c
        if (p.h_phase_err) p.h_phase_err[m] = perr - 4.0 * M_PI * p.fc * drift / c;
        const double v = p.v0 + p.accel * (double)m / p.prf;
        vel[m] = (double)std::llround(v * 10.0) * 0.1;   // navigation header, 0.1 m/s
        const double th = p.omega * (double)(m - M / 2) / p.prf;
        const double ct = std::cos(th), sn = std::sin(th);
        for (int k = 0; k < K; ++k) {
            const double R = p.r0_cells * cell + drift + sy[k] * ct + sx[k] * sn;
            const double A0 = -2.0 * p.fc * R / c + perr / (2.0 * M_PI) + ph0[k];
            const double A1 = -2.0 * (Kr * R - p.fc * v) / (c * p.Fs);
            const double A2 = 2.0 * Kr * v / (c * p.Fs * p.Fs);
            int64_t* q = &coef[((size_t)m * K + k) * 4];
            q[0] = frac64(A0);
            q[1] = frac64(A1);
            q[2] = frac64(A2);
            float a = (float)amp[k];
            int32_t ab;
            std::memcpy(&ab, &a, 4);
            q[3] = ab;
        }
    }
    if (h_vel)
        for (int m = 0; m < M; ++m) h_vel[m] = vel[m];
    const float scale = (float)(p.rms_counts / std::sqrt(pw > 0 ? pw : 1.0));
    const float nsig = (float)std::sqrt(pw / std::pow(10.0, p.snr_db / 10.0) / 2.0);
    cudaError_t e;
    if ((e = cudaMemcpyAsync(d_coef_scratch, coef.data(), coef.size() * sizeof(int64_t), cudaMemcpyHostToDevice, st)))
        return e;
    if (d_vel && (e = cudaMemcpyAsync(d_vel, vel.data(), M * sizeof(double), cudaMemcpyHostToDevice, st))) return e;
    dim3 g((N + 255) / 256, M);
    k_synth<<<g, 256, 4 * K * sizeof(int64_t), st>>>(d_coef_scratch, K, N, scale, nsig, p.seed * 0x9E37ull + 1, d_out);
    ISAR_COUNT(1);
    if ((e = cudaGetLastError())) return e;
    // the host vectors must outlive the asynchronous copies
    return cudaStreamSynchronize(st);
}

}  // namespace isar
