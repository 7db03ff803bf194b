"""ctypes bindings of the FP64 oracle (TEST INFRASTRUCTURE ONLY).

The oracle restates the reference's imaging chain on the CPU (isar_oracle.c).
Only tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU legs import
this package; the product (``isar_imaging_cuda_gb300``) never does.
"""
import ctypes as C
import os

import numpy as np

from . import build_oracle

_lib = None

STRETCH = 2
IFDS = 1
FLAG_HPC = 1
FLAG_MTRC = 2
FLAG_HRRP = 4


class Radar(C.Structure):
    _fields_ = [("echo_num", C.c_int), ("range_num", C.c_int),
                ("band_width", C.c_longlong), ("fc", C.c_longlong),
                ("Tp", C.c_double), ("Fs", C.c_longlong)]


class Trace(C.Structure):
    _fields_ = [("ra_shift", C.POINTER(C.c_double)),
                ("center_applied", C.c_int), ("center_shift", C.c_int),
                ("center_threshold", C.c_float),
                ("center_idx1_len", C.c_int), ("center_idx2_len", C.c_int),
                ("cut_offset", C.c_int), ("tgt_num", C.c_int),
                ("unit2_num", C.c_int), ("bins", C.c_int * 512),
                ("phase", C.c_void_p)]


class SynthCfg(C.Structure):
    _fields_ = [("M", C.c_int), ("N", C.c_int),
                ("fc", C.c_double), ("B", C.c_double), ("prf", C.c_double), ("Fs", C.c_double),
                ("n_scat", C.c_int), ("patch_x", C.c_double), ("patch_y", C.c_double),
                ("omega", C.c_double), ("r0_cells", C.c_double), ("drift_sigma", C.c_double),
                ("phase_uniform", C.c_double), ("phase_quad", C.c_double),
                ("v0", C.c_double), ("accel", C.c_double), ("snr_db", C.c_double),
                ("rms_counts", C.c_double), ("seed", C.c_uint64)]


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        _lib = C.CDLL(path)
        _lib.iso_image.restype = C.c_int
        _lib.iso_image.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(Radar), C.c_int, C.c_int,
                                   C.c_int, C.c_void_p, C.POINTER(Trace)]
        _lib.iso_synth.restype = None
        _lib.iso_synth.argtypes = [C.POINTER(SynthCfg), C.c_void_p, C.c_void_p]
        _lib.iso_fft.argtypes = [C.c_void_p, C.c_int, C.c_int]
        _lib.iso_fft.restype = C.c_int
        _lib.iso_image_entropy_f64.restype = C.c_double
        _lib.iso_image_entropy_f64.argtypes = [C.c_void_p, C.c_long]
        _lib.iso_image_entropy_f32.restype = C.c_double
        _lib.iso_image_entropy_f32.argtypes = [C.c_void_p, C.c_long]
        for name in ("iso_hpc", "iso_range_align", "iso_hrrp_center", "iso_cut",
                     "iso_fast_entropy", "iso_mtrc", "iso_post", "iso_doppler_tracking"):
            getattr(_lib, name).restype = None
        _lib.iso_cut.restype = C.c_int
        _lib.iso_next_pow2.restype = C.c_int
        _lib.iso_next_pow2.argtypes = [C.c_int]
        _lib.iso_hrrp.restype = None
        _lib.iso_hrrp.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int]
        _lib.iso_pulse_compress.restype = C.c_int
        _lib.iso_pulse_compress.argtypes = [C.c_void_p, C.c_int, C.c_double, C.POINTER(Radar), C.c_void_p]
    return _lib


def radar(M, N, B=1.0e9, fc=10.0e9, Fs=100.0e6, Tp=None):
    """RadarParameters for an M x N STRETCH frame (Tp defaults to N/Fs)."""
    if Tp is None:
        Tp = N / Fs
    return Radar(int(M), int(N), int(B), int(fc), float(Tp), int(Fs))


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def synth(cfg: dict):
    """Seeded synthetic STRETCH echoes -> (int16 iq [M,N,2], velocity [M])."""
    d = dict(fc=10e9, B=1e9, prf=1000.0, Fs=100e6, n_scat=50, patch_x=20.0, patch_y=20.0,
             omega=0.02, r0_cells=20.0, drift_sigma=0.3, phase_uniform=np.pi, phase_quad=0.0,
             v0=0.0, accel=0.0, snr_db=10.0, rms_counts=1000.0, seed=1)
    d.update(cfg)
    sc = SynthCfg(**{k: d[k] for k, _ in SynthCfg._fields_})
    iq = np.zeros((sc.M, sc.N, 2), np.int16)
    vel = np.zeros(sc.M, np.float64)
    lib().iso_synth(C.byref(sc), _ptr(iq), _ptr(vel))
    return iq, vel


def iq_to_c64(iq):
    """int16 I/Q -> complex64, as getSignalData's int16 -> float conversion."""
    return (iq[..., 0].astype(np.float32) + 1j * iq[..., 1].astype(np.float32)).astype(np.complex64)


def image(echo, velocity, rp: Radar, data_type=STRETCH, hpc=False, mtrc=False, iters=120, hrrp=False):
    """Runs the whole FP64 chain.  echo: complex64 [M,N].  Returns (img f64 [M,512], trace dict)."""
    M, N = rp.echo_num, rp.range_num
    e = np.ascontiguousarray(echo, np.complex64).view(np.float32).reshape(M, N, 2)
    v = np.ascontiguousarray(velocity if velocity is not None else np.zeros(M), np.float64)
    img = np.zeros((M, 512), np.float64)
    shifts = np.zeros(max(M - 1, 1), np.float64)
    phase = np.zeros(M, np.complex128)
    tr = Trace()
    tr.ra_shift = shifts.ctypes.data_as(C.POINTER(C.c_double))
    tr.phase = phase.ctypes.data
    flags = (FLAG_HPC if hpc else 0) | (FLAG_MTRC if mtrc else 0) | (FLAG_HRRP if hrrp else 0)
    rc = lib().iso_image(_ptr(e), _ptr(v), C.byref(rp), data_type, flags, iters, _ptr(img), C.byref(tr))
    if rc != 0:
        raise ValueError("oracle rejected the frame (rc=%d)" % rc)
    U = tr.unit2_num
    trace = dict(ra_shift=shifts[:M - 1].copy(), center_applied=tr.center_applied,
                 center_shift=tr.center_shift, center_threshold=tr.center_threshold,
                 center_idx1_len=tr.center_idx1_len, center_idx2_len=tr.center_idx2_len,
                 cut_offset=tr.cut_offset, tgt_num=tr.tgt_num, unit2_num=U,
                 bins=np.array(tr.bins[:min(U, 512)], np.int32), phase=phase)
    return img, trace


def entropy(img):
    a = np.ascontiguousarray(img)
    if a.dtype == np.float32:
        return lib().iso_image_entropy_f32(_ptr(a), a.size)
    a = np.ascontiguousarray(a, np.float64)
    return lib().iso_image_entropy_f64(_ptr(a), a.size)


# ---- stage-level access (each works on a complex128 copy) -----------------
def _c128(a):
    return np.ascontiguousarray(a, np.complex128)


def hpc(echo, velocity, rp: Radar):
    x = _c128(echo).copy()
    lib().iso_hpc(_ptr(x), _ptr(np.ascontiguousarray(velocity, np.float64)), C.byref(rp))
    return x


def range_align(x, rp: Radar):
    """rangeAlignmentParallel on spectra x -> (profiles, shifts[M-1])."""
    y = _c128(x).copy()
    sh = np.zeros(max(rp.echo_num - 1, 1), np.float64)
    lib().iso_range_align(_ptr(y), C.byref(rp), _ptr(sh))
    return y, sh[:rp.echo_num - 1]


def center_cut(y, rp: Radar, inter_length=30):
    """HRRPCenter + cutRangeProfile -> (centred profiles, cut [M,512], trace)."""
    z = _c128(y).copy()
    tr = Trace()
    lib().iso_hrrp_center(_ptr(z), C.byref(rp), inter_length, C.byref(tr))
    cut = np.zeros((rp.echo_num, 512), np.complex128)
    off = lib().iso_cut(_ptr(z), _ptr(cut), rp.echo_num, rp.range_num, 512)
    return z, cut, dict(center_applied=tr.center_applied, center_shift=tr.center_shift,
                        center_threshold=tr.center_threshold, center_idx1_len=tr.center_idx1_len,
                        center_idx2_len=tr.center_idx2_len, cut_offset=off)


def fast_entropy(cut, iters=120):
    """fastEntropy in place on a copy of cut [M,512] -> (cut, trace)."""
    z = _c128(cut).copy()
    M = z.shape[0]
    phase = np.zeros(M, np.complex128)
    tr = Trace()
    tr.phase = phase.ctypes.data
    lib().iso_fast_entropy(_ptr(z), M, 512, iters, C.byref(tr))
    U = tr.unit2_num
    return z, dict(tgt_num=tr.tgt_num, unit2_num=U, bins=np.array(tr.bins[:min(U, 512)], np.int32),
                   phase=phase)


def mtrc(cut, rp: Radar, data_type=STRETCH):
    z = _c128(cut).copy()
    lib().iso_mtrc(_ptr(z), C.byref(rp), data_type)
    return z


def post(cut, data_type=STRETCH):
    z = _c128(cut).copy()
    M = z.shape[0]
    img = np.zeros((M, 512), np.float64)
    lib().iso_post(_ptr(z), M, 512, data_type, _ptr(img))
    return img


# ---- IFDS ingest ------------------------------------------------------------
RANGE_NUM_IFDS_PC = 4096


def pulse_compress(ad, velocity, rp: Radar):
    """IFDS pulse compression (common.cu:583-604, 635-746).  ad: int16
    [P, 2*iq_len] (I, Q interleaved per pulse), velocity: [P].  Returns
    (complex128 [P, 4096], offsets [P])."""
    ad = np.ascontiguousarray(ad, np.int16)
    P, two_l = ad.shape
    out = np.zeros((P, RANGE_NUM_IFDS_PC), np.complex128)
    offs = np.zeros(P, np.int32)
    for p in range(P):
        row = np.ascontiguousarray(ad[p])
        o = np.zeros(RANGE_NUM_IFDS_PC, np.complex128)
        r = lib().iso_pulse_compress(_ptr(row), two_l // 2, float(velocity[p]), C.byref(rp), _ptr(o))
        if r < 0:
            raise ValueError("pulse compression rejected (iq_len %d)" % (two_l // 2))
        out[p] = o
        offs[p] = r
    return out, offs


def hrrp(echo, data_type=STRETCH):
    """getHRRP (common.cu:541-580): the M x N high-resolution range profiles
    of complex echoes [M, N] (complex128 result)."""
    x = _c128(echo)
    M, N = x.shape
    out = np.zeros((M, N), np.complex128)
    lib().iso_hrrp(_ptr(x), _ptr(out), M, N, int(data_type))
    return out
