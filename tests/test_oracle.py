"""CPU tests of the FP64 oracle: known-answer tests of its primitives."""
import ctypes as C

import numpy as np
import pytest

import oracle
from tests.helpers import make_frame


def test_next_pow2_matches_reference_semantics():
    # common.cu:521-529: 2^(floor(log2 n)+1), i.e. 2n for powers of two, 2 for 0
    lib = oracle.lib()
    for n, want in [(0, 2), (1, 2), (2, 4), (3, 4), (4, 8), (5, 8), (255, 256), (256, 512), (1023, 1024)]:
        assert lib.iso_next_pow2(n) == want


@pytest.mark.parametrize("n", [2, 8, 512, 4096])
@pytest.mark.parametrize("inverse", [0, 1])
def test_fft_vs_dft(n, inverse):
    rng = np.random.default_rng(n)
    x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex128)
    y = x.copy()
    oracle.lib().iso_fft(y.ctypes.data_as(C.c_void_p), n, inverse)
    want = np.fft.ifft(x) * n if inverse else np.fft.fft(x)
    assert np.max(np.abs(y - want)) <= 1e-10 * np.max(np.abs(want))


def test_synth_is_deterministic():
    a, va = make_frame(128, 512, seed=11)
    b, vb = make_frame(128, 512, seed=11)
    c, _ = make_frame(128, 512, seed=12)
    assert np.array_equal(a, b) and np.array_equal(va, vb)
    assert not np.array_equal(a, c)


def test_hpc_removes_injected_quadratic_phase():
    # a single scatterer with radial velocity: after HPC the row phase is linear in n
    M, N = 128, 512
    e, v = make_frame(M, N, seed=3, n_scat=1, snr_db=200.0, v0=3000.0, accel=50.0, drift_sigma=0.0,
                      phase_uniform=0.0)
    rp = oracle.radar(M, N)
    x = oracle.hpc(e, v, rp)
    ph = np.unwrap(np.angle(x[5]))
    n = np.arange(N)
    resid = ph - np.polyval(np.polyfit(n, ph, 1), n)
    ph0 = np.unwrap(np.angle(e[5].astype(np.complex128)))
    resid0 = ph0 - np.polyval(np.polyfit(n, ph0, 1), n)
    assert np.max(np.abs(resid)) < 0.05 < np.max(np.abs(resid0))


def test_range_align_recovers_injected_drift():
    # pure range drift (no rotation, no phase error): aligned profiles peak in one cell
    M, N = 128, 1024
    e, _ = make_frame(M, N, seed=5, n_scat=1, snr_db=60.0, omega=0.0, drift_sigma=0.8, phase_uniform=0.0)
    rp = oracle.radar(M, N)
    y, sh = oracle.range_align(e, rp)
    peaks = np.argmax(np.abs(y), axis=1)
    assert np.ptp(peaks) <= 1
    assert np.max(np.abs(sh)) > 0.5


def test_full_chain_focuses():
    M, N = 128, 512
    e, v = make_frame(M, N, seed=7)
    rp = oracle.radar(M, N)
    img, tr = oracle.image(e, v, rp)
    img0, _ = oracle.image(e, v, rp, iters=0)
    assert img.shape == (M, 512)
    assert oracle.entropy(img) <= oracle.entropy(img0) + 1e-9
    assert 2 <= tr["unit2_num"] <= 512 and tr["unit2_num"] == len(tr["bins"])
    assert np.all(np.diff(tr["bins"]) >= 0)
