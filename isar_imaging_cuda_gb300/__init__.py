"""GB300-native ISAR range-Doppler imaging (sm_103a).

Python view of ``libisar_gb300.so`` through its plain C ABI
(``include/isar_gb300.h``).  The library re-implements the imaging chain of
Junf137/isar_imaging_cuda behind ``isarMainSingle``: high-speed compensation,
range alignment, HRRP centering and cut, Doppler tracking + fast minimum
entropy autofocus, CZT MTRC correction and image formation.

Device buffers are passed as torch CUDA tensors (or raw integer device
pointers).  The CUDA library must be built (``build.build()``); there is no
CPU fallback: every call fails loudly when the extension is missing.
"""
import ctypes as C
import os

from . import build as _build

STRETCH = 2
IFDS = 1
FLAG_HPC = 1
FLAG_MTRC = 2
FLAG_HRRP = 4
FLAG_IQ16 = 8   # d_echo holds int16 I/Q samples (device buffers)
RANGE_NUM_CUT = 512

ISAR_OK = 0
_ERRORS = {-1: "EINVAL", -2: "ECUDA", -3: "ENOMEM", -4: "ESTATE", -5: "EIO"}

# every symbol the C headers declare with ISAR_API (checked by the tests)
EXPORTS = ("isar_get_last_error", "isar_version", "isar_create", "isar_destroy", "isar_stream",
           "isar_image_host", "isar_image_device", "isar_get_trace", "isar_stage_hpc",
           "isar_stage_range_align", "isar_stage_center_cut", "isar_stage_fast_entropy",
           "isar_stage_post", "isar_fft_rows", "isar_get_profiles", "isar_synth_device", "isar_launch_count",
           "isar_synchronize", "isar_set_ra_shifts", "isar_test_barrier_timeout", "isar_center_cut_noalloc",
           "isar_get_tuning",
           "isar_set_tuning", "isar_autotune", "isar_batch_create", "isar_batch_destroy", "isar_batch_stream",
           "isar_batch_run", "isar_batch_synchronize", "isar_batch_set_tuning", "isar_batch_get_tuning",
           "isar_batch_lanes", "isar_batch_autotune", "isar_wsnet_param_count", "isar_wsnet_create",
           "isar_wsnet_destroy", "isar_wsnet_stream", "isar_wsnet_set_params", "isar_wsnet_get_params",
           "isar_wsnet_forward", "isar_wsnet_backward", "isar_wsnet_get_grads", "isar_wsnet_adam",
           "isar_nn_gemm_bf16", "isar_set_warmstart", "isar_frame_features", "isar_batch_set_warmstart",
           "isar_pulse_compress", "isar_stage_hrrp", "isar_iq16_to_c64")


class IsarError(RuntimeError):
    pass


class Radar(C.Structure):
    """isar_radar: RadarParameters (common.cuh:96-117) + data type."""
    _fields_ = [("echo_num", C.c_int), ("range_num", C.c_int), ("band_width", C.c_longlong),
                ("fc", C.c_longlong), ("Tp", C.c_double), ("Fs", C.c_longlong), ("data_type", C.c_int)]


class SynthParams(C.Structure):
    _fields_ = [("M", C.c_int), ("N", C.c_int), ("fc", C.c_double), ("B", C.c_double), ("prf", C.c_double),
                ("Fs", C.c_double), ("n_scat", C.c_int), ("patch_x", C.c_double), ("patch_y", C.c_double),
                ("omega", C.c_double), ("r0_cells", C.c_double), ("drift_sigma", C.c_double),
                ("phase_uniform", C.c_double), ("phase_quad", C.c_double), ("v0", C.c_double),
                ("accel", C.c_double), ("snr_db", C.c_double), ("rms_counts", C.c_double), ("seed", C.c_uint64),
                ("phase_poly_order", C.c_int), ("phase_poly_sigma", C.c_double), ("h_phase_err", C.c_void_p)]


class Trace(C.Structure):
    _fields_ = [("ra_shift", C.c_void_p), ("phase", C.c_void_p), ("center_applied", C.c_int),
                ("center_shift", C.c_int), ("cut_offset", C.c_int), ("center_idx1_len", C.c_int),
                ("center_idx2_len", C.c_int), ("center_threshold", C.c_float), ("tgt_num", C.c_int),
                ("unit2_num", C.c_int), ("bins", C.c_int * 512), ("af_iterations", C.c_int),
                ("af_entropy", C.c_float), ("ws_used", C.c_int), ("af_entropy_final", C.c_float * 2),
                ("af_iterations_leg", C.c_int * 2)]


class Tuning(C.Structure):
    """isar_tuning: launch parameters of a context (defaults = the reference's)."""
    _fields_ = [("ra_pair_min", C.c_int), ("ra_rows_per_cta", C.c_int), ("ra_rows_final", C.c_int),
                ("af_cluster", C.c_int), ("af_tol", C.c_float), ("af_iters", C.c_int),
                ("af_cluster_max", C.c_int), ("ra_rows_each_level", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def lib_path():
    return _build.LIB


def load(build_if_missing=True):
    """Loads libisar_gb300.so (building it in-tree if missing)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise IsarError("libisar_gb300.so is not built (run isar_imaging_cuda_gb300.build.build())")
        _build.build()
    lib = C.CDLL(path)
    vp, i, d = C.c_void_p, C.c_int, C.c_double
    sig = {
        "isar_get_last_error": (i, [C.c_char_p, C.c_size_t]),
        "isar_version": (C.c_char_p, []),
        "isar_create": (i, [C.POINTER(vp), C.POINTER(Radar), i, vp]),
        "isar_destroy": (i, [vp]),
        "isar_stream": (vp, [vp]),
        "isar_image_host": (i, [vp, vp, vp, i, vp]),
        "isar_image_device": (i, [vp, vp, vp, i, vp]),
        "isar_get_trace": (i, [vp, C.POINTER(Trace)]),
        "isar_stage_hpc": (i, [vp, vp, vp]),
        "isar_stage_range_align": (i, [vp, vp, vp, i]),
        "isar_stage_center_cut": (i, [vp, vp, vp]),
        "isar_stage_fast_entropy": (i, [vp, vp, i]),
        "isar_stage_post": (i, [vp, vp, i, vp]),
        "isar_fft_rows": (i, [vp, vp, i, i, i]),
        "isar_pulse_compress": (i, [vp, vp, i, vp, i, vp, vp]),
        "isar_stage_hrrp": (i, [vp, vp, vp]),
        "isar_iq16_to_c64": (i, [vp, vp, C.c_size_t, vp]),
        "isar_get_profiles": (i, [vp, C.POINTER(vp)]),
        "isar_synth_device": (i, [C.POINTER(SynthParams), vp, vp, vp, vp]),
        "isar_launch_count": (C.c_longlong, []),
        "isar_synchronize": (i, [vp]),
        "isar_set_ra_shifts": (i, [vp, vp]),
        "isar_test_barrier_timeout": (i, [vp, C.c_uint, i]),
        "isar_center_cut_noalloc": (i, [vp, i, i, vp, vp]),
        "isar_get_tuning": (i, [vp, C.POINTER(Tuning)]),
        "isar_set_tuning": (i, [vp, C.POINTER(Tuning)]),
        "isar_autotune": (i, [vp, vp, vp, i, i, C.POINTER(Tuning)]),
        "isar_batch_create": (i, [C.POINTER(vp), i, vp, i]),
        "isar_batch_destroy": (i, [vp]),
        "isar_batch_stream": (vp, [vp]),
        "isar_batch_run": (i, [vp, vp, i]),
        "isar_batch_synchronize": (i, [vp]),
        "isar_batch_set_tuning": (i, [vp, C.POINTER(Radar), C.POINTER(Tuning)]),
        "isar_batch_get_tuning": (i, [vp, C.POINTER(Radar), C.POINTER(Tuning)]),
        "isar_batch_lanes": (i, [vp]),
        "isar_batch_autotune": (i, [vp, vp, i, C.POINTER(C.c_float)]),
        "isar_wsnet_param_count": (i, []),
        "isar_wsnet_create": (i, [C.POINTER(vp), i, i, i, vp]),
        "isar_wsnet_destroy": (i, [vp]),
        "isar_wsnet_stream": (vp, [vp]),
        "isar_wsnet_set_params": (i, [vp, vp]),
        "isar_wsnet_get_params": (i, [vp, vp]),
        "isar_wsnet_forward": (i, [vp, vp, i, i, vp]),
        "isar_wsnet_backward": (i, [vp, vp, i, i, C.POINTER(C.c_float)]),
        "isar_wsnet_get_grads": (i, [vp, vp]),
        "isar_wsnet_adam": (i, [vp, C.c_float]),
        "isar_nn_gemm_bf16": (i, [vp, i, vp, i, vp, i, i, i, i, i, vp]),
        "isar_set_warmstart": (i, [vp, vp]),
        "isar_frame_features": (i, [vp, vp, vp, i, vp, vp]),
        "isar_batch_set_warmstart": (i, [vp, vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def launch_count():
    """Kernels launched by the library so far."""
    return int(load().isar_launch_count())


def last_error():
    buf = C.create_string_buffer(1024)
    load().isar_get_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def _check(rc, what):
    if rc != ISAR_OK:
        raise IsarError("%s failed (%s): %s" % (what, _ERRORS.get(rc, rc), last_error()))


def _dptr(t):
    """Device pointer of a torch CUDA tensor (or an int)."""
    if t is None:
        return None
    if isinstance(t, int):
        return t
    if not t.is_cuda:
        raise IsarError("expected a CUDA tensor")
    if not t.is_contiguous():
        raise IsarError("expected a contiguous tensor")
    return t.data_ptr()


def radar(M, N, B=1.0e9, fc=10.0e9, Fs=100.0e6, Tp=None, data_type=STRETCH):
    """Radar parameters of an M x N frame (Tp defaults to N / Fs)."""
    if Tp is None:
        Tp = N / Fs
    return Radar(int(M), int(N), int(B), int(fc), float(Tp), int(Fs), int(data_type))


def synth_params(M, N, seed, full=False, **kw):
    """Seeded synthetic-frame parameters: the plain workload (50 scatterers in
    20 m x 20 m, 0.02 rad/s, drift 0.3 cell, uniform phase error, SNR 10 dB,
    no radial velocity) or, with full=True, the five-stage workload (200
    scatterers in 40 m x 40 m, 4 degrees over the aperture, 3000 m/s and
    50 m/s^2, drift 0.5 cell, quadratic + random phase error, SNR 5 dB)."""
    import math
    d = dict(fc=10e9, B=1e9, prf=1000.0, Fs=100e6, n_scat=50, patch_x=20.0, patch_y=20.0, omega=0.02,
             r0_cells=20.0, drift_sigma=0.3, phase_uniform=math.pi, phase_quad=0.0, v0=0.0, accel=0.0,
             snr_db=10.0, rms_counts=1000.0)
    if full:
        d.update(n_scat=200, patch_x=40.0, patch_y=40.0, omega=math.radians(4.0) / (M / 1000.0),
                 drift_sigma=0.5, phase_uniform=0.5, phase_quad=6.0, v0=3000.0, accel=50.0, snr_db=5.0)
    d.update(kw)
    return SynthParams(M=M, N=N, seed=seed, **d)


def iq16_to_c64(d_iq, d_echo, stream=None):
    """int16 I/Q pairs (device tensor, ... x 2) -> complex64 as float32 pairs
    (device tensor with the same number of elements), stream-ordered."""
    n = d_iq.numel() // 2
    if d_echo.numel() != 2 * n:
        raise IsarError("d_echo must hold %d floats" % (2 * n))
    _check(load().isar_iq16_to_c64(_dptr(d_iq), _dptr(d_echo), n, C.c_void_p(stream) if stream else None),
           "isar_iq16_to_c64")


def synth_device(p: SynthParams, d_out, d_vel=None, stream=None, phase_err=False):
    """Generates one frame on the device; returns the host velocities (numpy)
    and, with phase_err=True, also the injected per-pulse phase error (rad)."""
    import numpy as np
    hv = np.zeros(p.M, np.float64)
    pe = np.zeros(p.M, np.float64) if phase_err else None
    p.h_phase_err = pe.ctypes.data if phase_err else None
    _check(load().isar_synth_device(C.byref(p), _dptr(d_out), _dptr(d_vel), hv.ctypes.data,
                                    C.c_void_p(stream) if stream else None), "isar_synth_device")
    p.h_phase_err = None
    return (hv, pe) if phase_err else hv


class Context:
    """An imaging context (workspace + tables + stream) for M x N frames."""

    def __init__(self, rp: Radar, device=0, stream=None):
        self._lib = load()
        self.radar = rp
        self.M, self.N = rp.echo_num, rp.range_num
        h = C.c_void_p()
        s = C.c_void_p(stream) if stream else None
        _check(self._lib.isar_create(C.byref(h), C.byref(rp), device, s), "isar_create")
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._lib.isar_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def stream(self):
        return self._lib.isar_stream(self._h)

    def image_host(self, echo, velocity=None, flags=0):
        """echo: numpy complex64 [M, N]; returns float32 image [M, 512] (blocking)."""
        import numpy as np
        e = np.ascontiguousarray(echo, np.complex64)
        if e.shape != (self.M, self.N):
            raise IsarError("echo shape %s != (%d, %d)" % (e.shape, self.M, self.N))
        v = None if velocity is None else np.ascontiguousarray(velocity, np.float64)
        img = np.empty((self.M, RANGE_NUM_CUT), np.float32)
        _check(self._lib.isar_image_host(self._h, e.ctypes.data, None if v is None else v.ctypes.data, flags,
                                         img.ctypes.data), "isar_image_host")
        return img

    def image_device(self, d_echo, d_velocity, d_img, flags=0):
        _check(self._lib.isar_image_device(self._h, _dptr(d_echo), _dptr(d_velocity), flags, _dptr(d_img)),
               "isar_image_device")

    def set_ra_shifts(self, shifts=None):
        """Test hook: range alignment uses these M-1 shifts (None: its own)."""
        import numpy as np
        if shifts is None:
            _check(self._lib.isar_set_ra_shifts(self._h, None), "isar_set_ra_shifts")
            return
        self._given = np.ascontiguousarray(shifts, np.float32)
        _check(self._lib.isar_set_ra_shifts(self._h, self._given.ctypes.data), "isar_set_ra_shifts")

    def test_barrier_timeout(self, polls=0, never_complete=False):
        """Test hook: the autofocus grid barrier polls at most `polls` times
        and, with never_complete, waits for an arrival that never comes."""
        _check(self._lib.isar_test_barrier_timeout(self._h, int(polls), int(bool(never_complete))),
               "isar_test_barrier_timeout")

    def synchronize(self):
        _check(self._lib.isar_synchronize(self._h), "isar_synchronize")

    def profiles_ptr(self):
        p = C.c_void_p()
        _check(self._lib.isar_get_profiles(self._h, C.byref(p)), "isar_get_profiles")
        return p.value

    def trace(self):
        import numpy as np
        sh = np.zeros(self.M - 1, np.float32)
        ph = np.zeros(self.M, np.complex64)
        t = Trace()
        t.ra_shift = sh.ctypes.data
        t.phase = ph.ctypes.data
        _check(self._lib.isar_get_trace(self._h, C.byref(t)), "isar_get_trace")
        U = t.unit2_num
        return dict(ra_shift=sh, phase=ph, center_applied=t.center_applied, center_shift=t.center_shift,
                    cut_offset=t.cut_offset, center_idx1_len=t.center_idx1_len,
                    center_idx2_len=t.center_idx2_len, center_threshold=t.center_threshold,
                    tgt_num=t.tgt_num, unit2_num=U, bins=np.array(t.bins[:min(U, 512)], np.int32),
                    af_iterations=t.af_iterations, af_entropy=t.af_entropy, ws_used=t.ws_used,
                    af_entropy_final=(t.af_entropy_final[0], t.af_entropy_final[1]),
                    af_iterations_leg=(t.af_iterations_leg[0], t.af_iterations_leg[1]))

    def tuning(self):
        t = Tuning()
        _check(self._lib.isar_get_tuning(self._h, C.byref(t)), "isar_get_tuning")
        return t

    def set_tuning(self, **kw):
        """Updates the named isar_tuning fields, e.g. set_tuning(af_cluster=8)."""
        t = self.tuning()
        for k, v in kw.items():
            if not hasattr(t, k):
                raise KeyError(k)
            setattr(t, k, v)
        _check(self._lib.isar_set_tuning(self._h, C.byref(t)), "isar_set_tuning")
        return t

    # stage entry points (device buffers, stream-ordered)
    def stage_hpc(self, d_x, d_vel):
        _check(self._lib.isar_stage_hpc(self._h, _dptr(d_x), _dptr(d_vel)), "isar_stage_hpc")

    def stage_range_align(self, d_x, d_vel=None, flags=0):
        _check(self._lib.isar_stage_range_align(self._h, _dptr(d_x), _dptr(d_vel), flags),
               "isar_stage_range_align")

    def stage_center_cut(self, d_y, d_cut):
        _check(self._lib.isar_stage_center_cut(self._h, _dptr(d_y), _dptr(d_cut)), "isar_stage_center_cut")

    def stage_hrrp(self, d_x, d_hrrp):
        _check(self._lib.isar_stage_hrrp(self._h, _dptr(d_x), _dptr(d_hrrp)), "isar_stage_hrrp")

    def stage_fast_entropy(self, d_cut, iterations=120):
        _check(self._lib.isar_stage_fast_entropy(self._h, _dptr(d_cut), iterations), "isar_stage_fast_entropy")

    def stage_post(self, d_cut, d_img, flags=0):
        _check(self._lib.isar_stage_post(self._h, _dptr(d_cut), flags, _dptr(d_img)), "isar_stage_post")

    def fft_rows(self, d_x, rows, n, inverse=False):
        _check(self._lib.isar_fft_rows(self._h, _dptr(d_x), rows, n, 1 if inverse else 0), "isar_fft_rows")

    def pulse_compress(self, d_ad, iq_len, d_velocity, d_out, d_offsets=None):
        """IFDS pulse compression: d_ad int16 [P, 2*iq_len] (I, Q
        interleaved), d_velocity float64 [P], d_out float32 [P, 4096, 2],
        d_offsets int32 [P] or None (device tensors)."""
        P = d_velocity.shape[0]
        _check(self._lib.isar_pulse_compress(self._h, _dptr(d_ad), int(iq_len), _dptr(d_velocity), P,
                                             _dptr(d_out), _dptr(d_offsets)), "isar_pulse_compress")

    def autotune(self, d_echo, d_velocity=None, flags=0, engines=3):
        """isar_autotune: times frames of d_echo over the launch parameters,
        applies and returns the fastest isar_tuning."""
        t = Tuning()
        _check(self._lib.isar_autotune(self._h, _dptr(d_echo), _dptr(d_velocity), flags, engines, C.byref(t)),
               "isar_autotune")
        return t

    def features(self, d_echo, d_velocity, flags, d_x0, d_psi):
        """isar_frame_features: warm-start network inputs of one frame."""
        _check(self._lib.isar_frame_features(self._h, _dptr(d_echo), _dptr(d_velocity), flags, _dptr(d_x0),
                                             _dptr(d_psi)), "isar_frame_features")

    def set_warmstart(self, net):
        """Attaches a WSNet as the autofocus warm start (None detaches)."""
        _check(self._lib.isar_set_warmstart(self._h, net._h if net is not None else None), "isar_set_warmstart")
        self._ws = net


class WSNet:
    """The learned autofocus warm-start network (isar_wsnet_*)."""

    def __init__(self, max_rows, training=False, device=0, stream=None):
        self._lib = load()
        h = C.c_void_p()
        _check(self._lib.isar_wsnet_create(C.byref(h), int(max_rows), 1 if training else 0, device,
                                           C.c_void_p(stream) if stream else None), "isar_wsnet_create")
        self._h = h
        self.n_params = int(self._lib.isar_wsnet_param_count())

    @property
    def stream(self):
        return self._lib.isar_wsnet_stream(self._h)

    def set_params(self, p):
        import numpy as np
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.n_params
        _check(self._lib.isar_wsnet_set_params(self._h, p.ctypes.data), "isar_wsnet_set_params")

    def params(self):
        import numpy as np
        p = np.zeros(self.n_params, np.float32)
        _check(self._lib.isar_wsnet_get_params(self._h, p.ctypes.data), "isar_wsnet_get_params")
        return p

    def grads(self):
        import numpy as np
        g = np.zeros(self.n_params, np.float32)
        _check(self._lib.isar_wsnet_get_grads(self._h, g.ctypes.data), "isar_wsnet_get_grads")
        return g

    def forward(self, d_x0, frames, M, d_out=None):
        _check(self._lib.isar_wsnet_forward(self._h, _dptr(d_x0), frames, M, _dptr(d_out)), "isar_wsnet_forward")

    def backward(self, d_target, frames, M):
        loss = C.c_float()
        _check(self._lib.isar_wsnet_backward(self._h, _dptr(d_target), frames, M, C.byref(loss)),
               "isar_wsnet_backward")
        return loss.value

    def adam(self, lr):
        _check(self._lib.isar_wsnet_adam(self._h, C.c_float(lr)), "isar_wsnet_adam")

    def save(self, path):
        import numpy as np
        np.save(path, self.params())

    def load_params(self, path):
        import numpy as np
        self.set_params(np.load(path))

    def close(self):
        if getattr(self, "_h", None):
            self._lib.isar_wsnet_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def gemm_bf16(d_a, lda, d_b, ldb, d_c, ldc, M, N, K, splits=1, stream=None):
    """Tensor-core test GEMM: C[M][N] = A[M][K] B[N][K]^T (bf16 in, fp32 out)."""
    _check(load().isar_nn_gemm_bf16(_dptr(d_a), lda, _dptr(d_b), ldb, _dptr(d_c), ldc, M, N, K, splits,
                                    C.c_void_p(stream) if stream else None), "isar_nn_gemm_bf16")


WARMSTART_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights", "warmstart.npy")


class BatchFrame(C.Structure):
    """isar_batch_frame: one frame of a batch (device buffers)."""
    _fields_ = [("radar", Radar), ("d_echo", C.c_void_p), ("d_velocity", C.c_void_p), ("flags", C.c_int),
                ("d_img", C.c_void_p)]


class Batch:
    """Many frames of uneven size imaged by one CUDA graph (isar_batch_*)."""

    def __init__(self, device=0, stream=None, lanes=0):
        self._lib = load()
        h = C.c_void_p()
        _check(self._lib.isar_batch_create(C.byref(h), device, C.c_void_p(stream) if stream else None, lanes),
               "isar_batch_create")
        self._h = h

    @staticmethod
    def frames(items):
        """items: iterable of (radar, d_echo, d_velocity, flags, d_img)."""
        items = list(items)
        arr = (BatchFrame * len(items))()
        for k, (rp, e, v, fl, img) in enumerate(items):
            arr[k] = BatchFrame(rp, _dptr(e), _dptr(v), fl, _dptr(img))
        return arr

    def run(self, frames):
        _check(self._lib.isar_batch_run(self._h, frames, len(frames)), "isar_batch_run")

    def synchronize(self):
        _check(self._lib.isar_batch_synchronize(self._h), "isar_batch_synchronize")

    def autotune(self, frames):
        ms = C.c_float()
        _check(self._lib.isar_batch_autotune(self._h, frames, len(frames), C.byref(ms)), "isar_batch_autotune")
        return ms.value

    def lanes(self):
        return int(self._lib.isar_batch_lanes(self._h))

    def set_warmstart(self, net):
        """Attaches a WSNet as the warm start of every lane (None detaches)."""
        _check(self._lib.isar_batch_set_warmstart(self._h, net._h if net is not None else None),
               "isar_batch_set_warmstart")
        self._ws = net

    def set_tuning(self, rp, t):
        _check(self._lib.isar_batch_set_tuning(self._h, C.byref(rp), C.byref(t)), "isar_batch_set_tuning")

    def tuning(self, rp):
        t = Tuning()
        _check(self._lib.isar_batch_get_tuning(self._h, C.byref(rp), C.byref(t)), "isar_batch_get_tuning")
        return t

    @property
    def stream(self):
        return self._lib.isar_batch_stream(self._h)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.isar_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
