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
