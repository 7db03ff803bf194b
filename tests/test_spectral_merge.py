"""The identity behind the range-alignment spectral envelope merge, in numpy
(no GPU): the 2N-point spectrum of a row's half-cell power
w[2n] = |p(n)|^2, w[2n+1] = |p(n + 1/2)|^2 turns a shift of the row by s
cells (ramp exp(-j 2 pi k s / N) on its spectrum, k = 0..N-1, as the
reference's rangeAlignmentParallel applies it) into the phase ramp
exp(-j 2 pi d s / N) on the lag d, so a group's power envelope is the even-
sample inverse transform of the sum of its rows' shifted spectra (checked in
FP64).  The CUDA kernels k_ra_spec0 / k_ra_spec follow these steps in FP32;
a complex64 run of the whole formulation is checked against the FP64
oracle's shifts."""
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


def _f32_window(N):
    """hamming(n) * cos(pi n) in float as the reference forms it (the oracle's
    window up to the last rounding of cos)."""
    n = np.arange(N)
    f32 = np.float32
    ham = (f32(0.54) - f32(0.46) * np.cos((f32(2 * np.pi) * n.astype(f32)) / f32(N - 1)).astype(f32)).astype(f32)
    return (ham * np.cos((f32(np.pi) * n.astype(f32)).astype(np.float64)).astype(f32)).astype(f32)


def _f32_shift(a, b):
    """The pair shift as the range-alignment kernels compute it: complex64
    transforms locate the peak, the three parabola samples are exact sums,
    the parabola is fitted in float."""
    sf = pytest.importorskip("scipy.fft")
    f32 = np.float32
    N = a.shape[0]
    c = sf.ifft(sf.fft(a.astype(np.complex64)) * np.conj(sf.fft(b.astype(np.complex64)))).real
    pos = int(np.argmax(np.abs(np.roll(c, N // 2))))
    tau = (pos + N // 2) % N
    f = [f32(np.dot(a.astype(np.float64), np.roll(b.astype(np.float64), tau + j - 1))) for j in range(3)]
    fa = (f[0] + f[2] - f32(2) * f[1]) / f32(2)
    fb = (f[2] - f[0]) / f32(2)
    return f32(f32(pos) + (-fb / (f32(2) * fa))) - f32(N / 2)


def spectral_model_shifts(x, N):
    """The spectral envelope merge in complex64 arithmetic (the kernels'
    precision) on the HPC-compensated spectra x [M][N]: the per-(level, pair)
    shifts, level-major as isar_trace.ra_shift."""
    sf = pytest.importorskip("scipy.fft")
    M = x.shape[0]
    u = (x * _f32_window(N)[None, :] / N).astype(np.complex64)
    k = np.arange(N)
    p0 = sf.ifft(u, axis=1) * N
    p1 = sf.ifft((u * np.exp(1j * np.pi * k / N)).astype(np.complex64), axis=1) * N
    c = ((np.abs(p0) ** 2) + 1j * (np.abs(p1) ** 2)).astype(np.complex64)
    Z = sf.fft(c, axis=1)
    Zm = np.conj(Z[:, (-k) % N])
    W = ((Z + Zm) / 2 + np.exp(-1j * np.pi * k / N) * (Z - Zm) / 2j).astype(np.complex64)
    amp = np.abs(p0).astype(np.float32)
    got, G = [], []
    for j in range(M // 2):
        s = _f32_shift(amp[2 * j], amp[2 * j + 1])
        got.append(s)
        G.append((W[2 * j] + np.exp(-2j * np.pi * k * float(s) / N) * W[2 * j + 1]).astype(np.complex64))
    while len(G) > 1:
        nxt = []
        for Wa, Wb in zip(G[0::2], G[1::2]):
            X = [Wg + np.conj(Wg[(N - k) % N]) for Wg in (Wa, Wb)]
            for Xg, Wg in zip(X, (Wa, Wb)):
                Xg[0] = Wg[0]
            env = sf.ifft((X[0] + 1j * X[1]).astype(np.complex64)) * N / (2 * N)
            s = _f32_shift(np.sqrt(np.maximum(env.real, 0)).astype(np.float32),
                           np.sqrt(np.maximum(env.imag, 0)).astype(np.float32))
            got.append(s)
            nxt.append((Wa + np.exp(-2j * np.pi * k * float(s) / N) * Wb).astype(np.complex64))
        G = nxt
    return np.array(got, np.float64)


def _model_frame(M, N, full):
    import oracle
    from tests.helpers import make_frame
    e, v = make_frame(M, N, seed=M + N, full=full)
    rp = oracle.radar(M, N)
    x = oracle.hpc(e, v, rp) if full else e.astype(np.complex128)
    return e, v, x, rp


@pytest.mark.parametrize("M,N,full", [(128, 512, False), (256, 1024, True)])
def test_fp32_spectral_formulation_reproduces_the_oracle_shifts(M, N, full):
    """The spectral merge in complex64 arithmetic gives the FP64 oracle's
    range-alignment shifts on seeded frames."""
    import oracle
    _, _, x, rp = _model_frame(M, N, full)
    _, want = oracle.range_align(x, rp)
    got = spectral_model_shifts(x, N)
    assert np.max(np.abs(got - want)) < 2e-3


@pytest.mark.gpu
@pytest.mark.parametrize("M,N,full", [(128, 512, False), (256, 1024, True)])
def test_spectral_merge_kernels_follow_the_model(torch_cuda, gb300, M, N, full):
    """The range-alignment kernels of the spectral path (k_ra_spec0, k_ra_spec)
    against the complex64 model above: every per-level shift within 2e-3
    cell, and 99% within 1e-4 (they differ only where a correlation sample
    sits at a float rounding boundary).  This ties the kernels' own details
    (the d = 0 handling of the packed spectra, the half-cell ramps, the
    fixed-point phase ramps) to the model that is checked against the
    oracle."""
    torch = torch_cuda
    e, v, x, _ = _model_frame(M, N, full)
    model = spectral_model_shifts(x, N)
    d = torch.from_numpy(np.ascontiguousarray(e, np.complex64).view(np.float32).copy()).cuda()
    dv = torch.from_numpy(v).cuda()
    with gb300.Context(gb300.radar(M, N), stream=torch.cuda.current_stream().cuda_stream) as ctx:
        ctx.set_tuning(ra_rows_each_level=0)
        ctx.stage_range_align(d, dv, gb300.FLAG_HPC if full else 0)
        got = ctx.trace()["ra_shift"].astype(np.float64)
    diff = np.abs(got - model)
    assert diff.max() < 2e-3, diff.max()
    assert np.mean(diff <= 1e-4) >= 0.99, np.sort(diff)[-5:]
