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
    int phase_poly_order;      // >= 2: random polynomial phase error of this order
    double phase_poly_sigma;   // rad, coefficient spread
    double* h_phase_err;       // out: M doubles or nullptr
};

cudaError_t synth_frame(const SynthParams& p, float2* d_out, double* d_vel, double* h_vel, int64_t* d_coef_scratch,
                        cudaStream_t st);

}  // namespace isar
