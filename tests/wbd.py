"""Writer of synthetic .wbd radar files (test helper).

Layout read by the reference's ingest (common.cu:796-899, :1085-1100): every
frame is frame_len = 4*N + 256 bytes; bytes 0..143 of the first frame hold
uint32[36] with [4] = frame_len/4, [12] = fc MHz, [13] = B MHz, [15] = Tp us,
[17] = Fs MHz; bytes 48..91 of each frame hold uint32[11] navigation data
with [7] = range*10, [8] = velocity*10 (two's complement), [9]/[10] =
azimuth/pitching * 2^24/360 (two's complement); the int16 I/Q payload starts
at byte 256.
"""
import os

import numpy as np


def write_wbd(path, iq, velocity, fc=10e9, B=1e9, Tp=16e-6, Fs=128e6, range_m=None, azimuth=None, pitching=None):
    P, N, _ = iq.shape
    frame_len = 4 * N + 256
    rng = np.full(P, 1000.0) if range_m is None else np.asarray(range_m)
    az = np.linspace(10.0, 10.5, P) if azimuth is None else np.asarray(azimuth)
    pit = np.full(P, 5.0) if pitching is None else np.asarray(pitching)
    with open(path, "wb") as f:
        for p in range(P):
            h = np.zeros(64, np.uint32)
            h[4] = frame_len // 4
            h[12] = int(round(fc / 1e6))
            h[13] = int(round(B / 1e6))
            h[15] = int(round(Tp * 1e6))
            h[17] = int(round(Fs / 1e6))
            h[19] = int(round(rng[p] * 10))
            h[20] = np.int64(int(round(velocity[p] * 10))) & 0xFFFFFFFF
            h[21] = np.int64(int(round(az[p] * (1 << 24) / 360.0))) & 0xFFFFFFFF
            h[22] = np.int64(int(round(pit[p] * (1 << 24) / 360.0))) & 0xFFFFFFFF
            f.write(h.tobytes())
            f.write(np.ascontiguousarray(iq[p], np.int16).tobytes())
    return frame_len


def dropin_dir(root, name):
    d = os.path.join(root, name)
    os.makedirs(d, exist_ok=True)
    return d


# Ingest scenario shared by the golden generator and the ingest tests: one
# .wbd file of 200 pulses x 512 range cells whose pitching jumps by more than
# 0.2 degrees twice, so the turn-angle curve (common.cu:902-972) has three
# blocks of 45, 15 and 140 pulses (blocks of 21..39 pulses are avoided: the
# reference's interpolation then reads before its knot vector).
INGEST_P, INGEST_N = 200, 512


def write_ingest_scenario(d, data_type=2, seed=5):
    """Writes the scenario into directory d (emptied first); returns the file
    path.  STRETCH files end in 00_1101.wbd, IFDS files in 01_1101.wbd."""
    import oracle
    for f in os.listdir(d):
        os.remove(os.path.join(d, f))
    P, N = INGEST_P, INGEST_N
    cfg = dict(M=P, N=N, seed=seed, Fs=128e6, n_scat=30, v0=250.0, accel=-40.0)
    iq, vel = oracle.synth(cfg)
    pit = np.concatenate([np.full(45, 5.0), np.full(15, 5.5), np.full(140, 6.0)])
    # azimuth: slow drift in the long blocks (their knots are 20 pulses
    # apart), 0.1 degree steps in the 15-pulse block, whose curve steps
    # pulse by pulse (smaller steps make the float cosine of the angle round
    # to 1 or above, and the reference's acos then gives 0 or NaN)
    az = np.concatenate([np.linspace(10.0, 10.2, 45), 10.2 + 0.1 * np.arange(1, 16), 11.7 + 0.01 * np.arange(1, 141)])
    rng = np.linspace(1000.0, 1011.9, P)
    name = "syn_000004_1383_%s_1101.wbd" % ("00" if data_type == 2 else "01")
    path = os.path.join(d, name)
    write_wbd(path, iq, vel, Fs=128e6, Tp=16e-6, range_m=rng, azimuth=az, pitching=pit)
    return path
