"""Generates the golden vectors under tests/golden/ from the reference itself.

The reference's own sources (Junf137/isar_imaging_cuda/isar_imaging) are
compiled for the CPU by oracle/ref_emu (its kernels run as host loops, Thrust
on its CPP backend, cuFFT/cuBLAS calls on double-precision stand-ins) and
driven through its exports (imagingMemInit + isarMainSingle) on seeded
synthetic STRETCH frames.  Each fixture stores the int16 input, the radar
parameters and the reference's outputs: the final image and the M x 512 cut
after HRRPCenter + cutRangeProfile.  The pc_* fixtures hold seeded IFDS pulses
(int16 I/Q, velocities, radar parameters) and the reference's pulse
compression of each (its pulseCompression class, 4096 cells per pulse); the
hrrp_* fixtures hold seeded int16 frames and the reference's getHRRP of them;
the ingest_* fixtures hold what the reference's dataParsing / dataExtracting
return on the .wbd scenario of tests/wbd.py.

Run here (where the reference checkout is present):
    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
# the reference checkout whose sources the emulation compiles in place
os.environ.setdefault("ISAR_REFERENCE_DIR", "/root/reference/isar_imaging")

import oracle  # noqa: E402
from oracle import ref_emu  # noqa: E402
from tests.helpers import CFG_FULL, CFG_PLAIN, PC_CASES, full_omega, iq_checksum, make_ifds_pulses  # noqa: E402

FIXTURES = {
    # name: (M, N, full pipeline (HPC + MTRC), seed)
    "plain_256x1024": (256, 1024, False, 101),
    "full_256x1024": (256, 1024, True, 102),
    # the larger frames store their synthesis seed and a checksum of the
    # int16 samples instead of the samples (tests regenerate them with the
    # oracle's synthesis and check the checksum), and the image only
    "full_512x4096": (512, 4096, True, 103),
    "full_1024x8192": (1024, 8192, True, 41),
}
STORE_SAMPLES_UP_TO = 256 * 1024


def make(name):
    M, N, full, seed = FIXTURES[name]
    cfg = dict(CFG_FULL if full else CFG_PLAIN)
    if full:
        cfg["omega"] = full_omega(M)
    cfg.update(M=M, N=N, seed=seed)
    iq, vel = oracle.synth(cfg)
    echo = oracle.iq_to_c64(iq)
    out = ref_emu.frame(echo, vel, M, N, hpc=full, mtrc=full, checkpoints=True)
    path = os.path.join(HERE, name + ".npz")
    common = dict(velocity=vel, M=M, N=N, B=1e9, fc=10e9, Fs=100e6, Tp=N / 100e6, hpc=full, mtrc=full,
                  img=out["img"])
    if M * N <= STORE_SAMPLES_UP_TO:
        np.savez_compressed(path, iq=iq, cut=out["cut"], **common)
    else:
        np.savez_compressed(path, seed=seed, iq_checksum=iq_checksum(iq), **common)
    return path


def make_pc(name, P=3, seed=7):
    """IFDS pulse compression by the reference's pulseCompression class."""
    iq_len, Fs, Tp, B, fc = PC_CASES[name]
    ad, vel = make_ifds_pulses(P, iq_len, Fs, Tp, B, seed)
    out = ref_emu.pulse_compress(ad, vel, B, fc, Tp, Fs)
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, ad=ad, velocity=vel, iq_len=iq_len, Fs=Fs, Tp=Tp, B=B, fc=fc, out=out)
    return path


HRRP_CASES = {
    # name: (M, N, data_type 2 STRETCH / 1 IFDS, seed)
    "hrrp_stretch_16x1024": (16, 1024, 2, 31),
    "hrrp_ifds_8x4096": (8, 4096, 1, 32),
}


def make_hrrp(name):
    """getHRRP by the reference on seeded int16 I/Q frames (a few strong
    range cells over noise)."""
    M, N, dt, seed = HRRP_CASES[name]
    rng = np.random.default_rng(seed)
    x = rng.normal(0, 30, (M, N)) + 1j * rng.normal(0, 30, (M, N))
    n = np.arange(N)
    for _ in range(4):
        x += 500 * np.exp(2j * np.pi * (rng.uniform(0, N) * n / N + rng.uniform()))
    iq = np.clip(np.rint(np.stack([x.real, x.imag], -1)), -32768, 32767).astype(np.int16)
    out = ref_emu.hrrp(oracle.iq_to_c64(iq), dt)
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, iq=iq, data_type=dt, out=out)
    return path


INGEST_CASES = {
    # name: (data_type, extract window (window_len, window_head, sampling_stride) or None)
    "ingest_stretch": (2, (128, 30, 1)),
    "ingest_ifds": (1, None),
}


def make_ingest(name):
    """The reference's dataParsing (nav decode, turn-angle curve) and, for
    STRETCH, one dataExtracting (uniform sampling, int16 samples to float)
    on the .wbd scenario of tests/wbd.py (regenerated by the tests)."""
    import tempfile
    from tests.wbd import write_ingest_scenario
    dt, win = INGEST_CASES[name]
    with tempfile.TemporaryDirectory() as d:
        write_ingest_scenario(d, data_type=dt)
        fl, fn, dn, ta = ref_emu.parse(d, data_type=dt)
        extra = {}
        if win is not None:
            sn, dno, tao, dw = ref_emu.extract(d, *win, data_type=dt)
            extra = dict(window=np.array(win, np.int32), sn=sn, dataNOut=dno, turnAngleOut=tao, dataW=dw)
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, data_type=dt, frame_len=fl, frame_num=fn, dataN=dn, turnAngle=ta, **extra)
    return path


if __name__ == "__main__":
    for n in sys.argv[1:] or list(FIXTURES) + list(PC_CASES) + list(HRRP_CASES) + list(INGEST_CASES):
        print(make_pc(n) if n in PC_CASES else make_hrrp(n) if n in HRRP_CASES else
              make_ingest(n) if n in INGEST_CASES else make(n))
