"""The identity behind the shortened MTRC chain (csrc/mtrc.cu, k_czt with
the column correction): after the CZT, the reference's column
shift-IFFT-shift (mtrc.cu:53-61), row FFT + shift (:63-66; IFDS fliplr
:72-75), column fftshift (:69), window on row 0 (isar_main.cu:192, factor
hamming[c / M] for column c), column FFT + shift (:193-201; IFDS flipud
:201-204) and magnitude equal |row FFT of (a - (1 - hamming[0]) mean(a))|
when every column gets the same window factor, i.e. M >= 512 with 512
columns.  Checked here in FP64 with numpy's FFTs on random data; the GPU
tests compare the kernels with the oracle."""
import numpy as np
import pytest

C = 512


def literal(a, ham, ifds):
    M = a.shape[0]
    b = np.fft.fftshift(np.fft.ifft(np.fft.ifftshift(a, axes=0), axis=0), axes=0)
    d = np.fft.fftshift(np.fft.fft(b, axis=1), axes=1)
    if ifds:
        d = d[:, ::-1]
    x = np.roll(d, -M // 2, axis=0).copy()
    x[0, :] *= ham[np.arange(C) // M]
    y = np.fft.fftshift(np.fft.fft(x, axis=0), axes=0)
    if ifds:
        y = y[::-1, :]
    return np.abs(y)


def shortcut(a, ham, ifds):
    e = a - (1.0 - ham[0]) * a.mean(axis=0, keepdims=True)
    if ifds:
        e = e[::-1, :]
    r = np.fft.fftshift(np.fft.fft(e, axis=1), axes=1)
    if ifds:
        r = r[:, ::-1]
    return np.abs(r)


def hamming(M):
    return 0.54 - 0.46 * np.cos(2.0 * np.pi * np.arange(M) / (M - 1))


@pytest.mark.parametrize("M", [512, 1024])
@pytest.mark.parametrize("ifds", [False, True])
def test_column_chain_collapses_to_a_mean_correction(M, ifds):
    rng = np.random.default_rng(M + ifds)
    a = rng.standard_normal((M, C)) + 1j * rng.standard_normal((M, C)) + 2.0
    want = literal(a, hamming(M), ifds)
    got = shortcut(a, hamming(M), ifds)
    assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-12


@pytest.mark.parametrize("M", [128, 256])
def test_below_512_pulses_the_window_differs_between_columns(M):
    # why the kernels keep the full chain there: hamming[c / M] takes
    # 512 / M different values across the columns
    rng = np.random.default_rng(M)
    a = rng.standard_normal((M, C)) + 1j * rng.standard_normal((M, C)) + 2.0
    want = literal(a, hamming(M), False)
    got = shortcut(a, hamming(M), False)
    assert np.linalg.norm(got - want) / np.linalg.norm(want) > 1e-6
