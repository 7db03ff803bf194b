"""IFDS pulse compression on the GPU (isar_pulse_compress) against the
reference's own pulseCompression class (golden fixtures pc_*.npz, made by
tests/golden/make_golden.py from the reference's sources run on the CPU) and
the FP64 oracle: same 4096-cell cut offset for every pulse (exact), cut
within 1e-4 relative L2 (float FFTs and float chirp phases of up to ~2400
rad, whose rounding the reference shares)."""
import glob
import os

import numpy as np
import pytest

import oracle
from tests.helpers import PC_CASES, make_ifds_pulses, rel_l2

pytestmark = pytest.mark.gpu

PC_GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "pc_*.npz")))


def _compress(torch, g, ad, vel, iq_len, B, fc, Tp, Fs):
    rp = g.radar(128, 4096, B=B, fc=fc, Fs=Fs, Tp=Tp, data_type=g.IFDS)
    d_ad = torch.from_numpy(np.ascontiguousarray(ad, np.int16)).cuda()
    d_v = torch.from_numpy(np.ascontiguousarray(vel, np.float64)).cuda()
    P = ad.shape[0]
    out = torch.full((P, 4096, 2), np.nan, dtype=torch.float32, device="cuda")
    offs = torch.full((P,), -1, dtype=torch.int32, device="cuda")
    with g.Context(rp, stream=torch.cuda.current_stream().cuda_stream) as ctx:
        ctx.pulse_compress(d_ad, iq_len, d_v, out, offs)
        ctx.synchronize()
    o = out.cpu().numpy()
    return (o[..., 0] + 1j * o[..., 1]).astype(np.complex64), offs.cpu().numpy()


@pytest.mark.parametrize("path", PC_GOLDEN, ids=[os.path.basename(p)[:-4] for p in PC_GOLDEN])
def test_pulse_compression_matches_reference_golden(torch_cuda, gb300, path):
    z = np.load(path)
    got, offs = _compress(torch_cuda, gb300, z["ad"], z["velocity"], int(z["iq_len"]), float(z["B"]),
                          float(z["fc"]), float(z["Tp"]), float(z["Fs"]))
    rp = oracle.Radar(0, 4096, int(float(z["B"])), int(float(z["fc"])), float(z["Tp"]), int(float(z["Fs"])))
    want, woffs = oracle.pulse_compress(z["ad"], z["velocity"], rp)
    assert np.array_equal(offs, woffs)
    for p in range(got.shape[0]):
        assert rel_l2(got[p], z["out"][p]) < 1e-4, p
        assert rel_l2(got[p], want[p]) < 1e-4, p


def test_pulse_compression_batch_of_many_pulses(torch_cuda, gb300):
    """A 64-pulse batch at NFFT 8192 (one launch): every pulse equals the
    oracle, and a repeated call (scratch reused) gives the same bits."""
    iq_len, Fs, Tp, B, fc = PC_CASES["pc_8192"]
    ad, vel = make_ifds_pulses(64, iq_len, Fs, Tp, B, seed=21)
    got, offs = _compress(torch_cuda, gb300, ad, vel, iq_len, B, fc, Tp, Fs)
    again, offs2 = _compress(torch_cuda, gb300, ad, vel, iq_len, B, fc, Tp, Fs)
    assert np.array_equal(got, again) and np.array_equal(offs, offs2)
    rp = oracle.Radar(0, 4096, int(B), int(fc), float(Tp), int(Fs))
    want, woffs = oracle.pulse_compress(ad, vel, rp)
    assert np.array_equal(offs, woffs)
    assert max(rel_l2(got[p], want[p]) for p in range(64)) < 1e-4


def test_pulse_compression_rejects_unsupported_lengths(torch_cuda, gb300):
    torch = torch_cuda
    rp = gb300.radar(128, 4096, B=50e6, fc=10e9, Fs=100e6, Tp=10e-6, data_type=gb300.IFDS)
    d_v = torch.zeros(2, dtype=torch.float64, device="cuda")
    out = torch.zeros((2, 4096, 2), dtype=torch.float32, device="cuda")
    with gb300.Context(rp, stream=torch.cuda.current_stream().cuda_stream) as ctx:
        for iq_len in (1000, 20000):   # NFFT 1024 (< 4096), 32768 (> 16384)
            d_ad = torch.zeros((2, 2 * iq_len), dtype=torch.int16, device="cuda")
            with pytest.raises(gb300.IsarError, match="nextPow2"):
                ctx.pulse_compress(d_ad, iq_len, d_v, out)
