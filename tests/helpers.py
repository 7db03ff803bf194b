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


def iq_checksum(iq):
    """Order-sensitive checksum of int16 samples: (sum, sum of index * value)."""
    a = np.asarray(iq, np.int64).ravel()
    return np.array([a.sum(), (a * (np.arange(a.size, dtype=np.int64) % 65521)).sum()], np.int64)


def golden_echo(z):
    """The complex64 input of a golden fixture: its stored int16 samples, or,
    for the larger fixtures, the frame regenerated from its seed by the
    oracle's synthesis (checked against the stored checksum)."""
    if "iq" in z:
        return oracle.iq_to_c64(z["iq"])
    M, N, seed, full = int(z["M"]), int(z["N"]), int(z["seed"]), bool(z["hpc"])
    cfg = dict(CFG_FULL if full else CFG_PLAIN)
    if full:
        cfg["omega"] = full_omega(M)
    cfg.update(M=M, N=N, seed=seed)
    iq, vel = oracle.synth(cfg)
    assert np.array_equal(iq_checksum(iq), z["iq_checksum"]), "synthesis differs from the fixture's"
    assert np.array_equal(vel, z["velocity"])
    return oracle.iq_to_c64(iq)


def rel_l2(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


# IFDS pulse-compression cases: (iq_len, Fs, Tp, B, fc); NFFT = nextPow2(iq_len)
# is 4096, 8192 (iq_len a power of two: the doubled NFFT of nextPow2) and 16384.
PC_CASES = {
    "pc_4096": (3000, 100e6, 10e-6, 50e6, 10e9),
    "pc_8192": (4096, 200e6, 10e-6, 100e6, 10e9),
    "pc_16384": (10000, 400e6, 10e-6, 300e6, 10e9),
}


def make_ifds_pulses(P, iq_len, Fs, Tp, B, seed, n_scat=3, amp=800.0, noise=40.0):
    """Seeded IFDS echoes: each pulse is the sum of n_scat delayed copies of
    the transmitted LFM chirp (Fs*Tp samples, rate B/Tp) with random complex
    amplitudes, plus complex Gaussian noise, as int16 [P, 2*iq_len] (I, Q
    interleaved); velocities in m/s [P]."""
    rng = np.random.default_rng(seed)
    S = int(Fs * Tp)
    t = (np.arange(S) - (S - 1) / 2.0) / Fs
    chirp = np.exp(1j * np.pi * B / Tp * t * t)
    ad = np.zeros((P, 2 * iq_len), np.int16)
    for p in range(P):
        x = (rng.normal(0, noise, iq_len) + 1j * rng.normal(0, noise, iq_len)).astype(np.complex128)
        for _ in range(n_scat):
            d = int(rng.integers(0, iq_len - S))
            a = amp * rng.uniform(0.3, 1.0) * np.exp(2j * np.pi * rng.uniform())
            x[d:d + S] += a * chirp
        q = np.clip(np.rint(np.stack([x.real, x.imag], -1)), -32768, 32767).astype(np.int16)
        ad[p] = q.reshape(-1)
    vel = rng.uniform(-300.0, 300.0, P)
    return ad, vel
