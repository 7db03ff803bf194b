// Synthetic echo generator interface (internal).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace isar {

struct SynthParams {
    int M, N;
    double fc, B, prf, Fs;
    int n_scat;
    double patch_x, patch_y, omega, r0_cells, drift_sigma, phase_uniform, phase_quad, v0, accel, snr_db, rms_counts;
    uint64_t seed;
};

cudaError_t synth_frame(const SynthParams& p, float2* d_out, double* d_vel, double* h_vel, int64_t* d_coef_scratch,
                        cudaStream_t st);

}  // namespace isar
