"""Shared helpers for the parity tests (test infrastructure)."""
import numpy as np

import oracle

# Synthetic workloads (seeded).  fc = 10 GHz, B = 1 GHz, PRF = 1 kHz, Fs = 100 MHz,
# Tp = N / Fs (one range cell = 0.15 m).
CFG_PLAIN = dict(n_scat=50, patch_x=20.0, patch_y=20.0, omega=0.02, drift_sigma=0.3,
                 phase_uniform=np.pi, phase_quad=0.0, v0=0.0, accel=0.0, snr_db=10.0)
CFG_FULL = dict(n_scat=200, patch_x=40.0, patch_y=40.0, drift_sigma=0.5, phase_uniform=0.5,
                phase_quad=6.0, v0=3000.0, accel=50.0, snr_db=5.0)


def full_omega(M, prf=1000.0, total_deg=4.0):
    return np.deg2rad(total_deg) / (M / prf)


def make_frame(M, N, seed, full=False, **kw):
    cfg = dict(CFG_FULL if full else CFG_PLAIN)
    if full:
        cfg["omega"] = full_omega(M)
    cfg.update(kw)
    cfg.update(M=M, N=N, seed=seed)
    iq, vel = oracle.synth(cfg)
    return oracle.iq_to_c64(iq), vel


def rel_l2(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
