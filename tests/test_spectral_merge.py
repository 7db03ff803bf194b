"""The identity behind the range-alignment spectral envelope merge, in FP64
numpy (no GPU): the 2N-point spectrum of a row's half-cell power
w[2n] = |p(n)|^2, w[2n+1] = |p(n + 1/2)|^2 turns a shift of the row by s
cells (ramp exp(-j 2 pi k s / N) on its spectrum, k = 0..N-1, as the
reference's rangeAlignmentParallel applies it) into the phase ramp
exp(-j 2 pi d s / N) on the lag d, so a group's power envelope is the even-
sample inverse transform of the sum of its rows' shifted spectra.  The CUDA
kernels k_ra_spec0 / k_ra_spec follow these steps in FP32."""
import numpy as np
import pytest


def half_cell_powers(u):
    """c[n] = w[2n] + j w[2n+1] for a row spectrum u (p = IFFT(u), unnormalised)."""
    N = u.shape[-1]
    k = np.arange(N)
    p0 = np.fft.ifft(u) * N
    p1 = np.fft.ifft(u * np.exp(1j * np.pi * k / N)) * N
    return np.abs(p0) ** 2 + 1j * np.abs(p1) ** 2


def power_spectrum(c):
    """W[d], d in [0, N), of the 2N-point real sequence w from one N-point FFT
    of w_even + j w_odd: W = E + exp(-j pi d / N) O."""
    N = c.shape[-1]
    d = np.arange(N)
    Z = np.fft.fft(c)
    Zm = np.conj(Z[(-d) % N])
    E, O = (Z + Zm) / 2, (Z - Zm) / 2j
    return E + np.exp(-1j * np.pi * d / N) * O


def envelope(W):
    """Even samples of the inverse 2N-point transform of the Hermitian W
    (only d in [0, N) kept, W[N] = 0): IFFT(W[d] + conj W[N - d]) / 2."""
    N = W.shape[-1]
    d = np.arange(N)
    X = W + np.conj(W[(N - d) % N])
    X[0] = W[0]
    return (np.fft.ifft(X) * N / (2 * N)).real


def shifted(u, s):
    N = u.shape[-1]
    return u * np.exp(-2j * np.pi * np.arange(N) * s / N)


@pytest.mark.parametrize("N", [64, 512, 2048])
def test_half_cell_spectrum_is_the_2n_point_fft(N):
    rng = np.random.default_rng(N)
    u = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    c = half_cell_powers(u)
    w = np.empty(2 * N)
    w[0::2], w[1::2] = c.real, c.imag
    full = np.fft.fft(w)
    W = power_spectrum(c)
    assert np.allclose(W, full[:N], rtol=0, atol=1e-9 * np.abs(full).max())
    assert abs(full[N]) < 1e-9 * np.abs(full).max()      # no lag of N


@pytest.mark.parametrize("N", [64, 1024])
def test_shift_is_a_lag_ramp(N):
    rng = np.random.default_rng(7 + N)
    u = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    d = np.arange(N)
    for s in (0.37, -5.25, 13.0, 0.5):
        want = power_spectrum(half_cell_powers(shifted(u, s)))
        got = power_spectrum(half_cell_powers(u)) * np.exp(-2j * np.pi * d * s / N)
        assert np.allclose(got, want, rtol=0, atol=1e-9 * np.abs(want).max())


def test_binary_merge_envelopes_match_direct_sums():
    """Three levels of the binary merge with fractional shifts: the envelope of
    every group from merged spectra equals the sum of its rows' powers at
    their cumulative shifts."""
    N, M = 256, 8
    rng = np.random.default_rng(3)
    U = rng.standard_normal((M, N)) + 1j * rng.standard_normal((M, N))
    d = np.arange(N)
    S = np.zeros(M)
    groups = [(power_spectrum(half_cell_powers(U[m])), [m]) for m in range(M)]
    while len(groups) > 1:
        nxt = []
        for (Wa, ra), (Wb, rb) in zip(groups[0::2], groups[1::2]):
            for Wg, rows in ((Wa, ra), (Wb, rb)):
                direct = sum(np.abs(np.fft.ifft(shifted(U[m], S[m])) * N) ** 2 for m in rows)
                assert np.allclose(envelope(Wg), direct, rtol=0, atol=1e-9 * direct.max())
            s = rng.uniform(-20, 20)
            S[rb] += s
            nxt.append((Wa + np.exp(-2j * np.pi * d * s / N) * Wb, ra + rb))
        groups = nxt
    Wg, rows = groups[0]
    direct = sum(np.abs(np.fft.ifft(shifted(U[m], S[m])) * N) ** 2 for m in rows)
    assert np.allclose(envelope(Wg), direct, rtol=0, atol=1e-9 * direct.max())
