"""Bounded device waits (the replacement for the reference's exit() on a CUDA
error, helper_cuda.h:583-595, and its fixed-count loops): the cooperative
autofocus engine's grid barrier is made to wait for an arrival that never
comes (a test hook of the C ABI) with a short poll limit.  Every CTA gives up,
sets the timeout flag and leaves the kernel; the frame reports ISAR_ECUDA
through the C ABI, and the next frame on the same context is imaged normally,
bit for bit as before.  No GPU fault, trap or endless loop is involved."""
import time

import numpy as np
import pytest

from tests.helpers import make_frame

pytestmark = pytest.mark.gpu

ISAR_ECUDA = -2


def test_grid_barrier_timeout_reports_ecuda_and_the_context_stays_usable(torch_cuda, gb300):
    torch = torch_cuda
    M, N = 256, 1024
    e, v = make_frame(M, N, seed=61)
    lib = gb300.load()
    with gb300.Context(gb300.radar(M, N)) as ctx:
        ctx.set_tuning(af_cluster=0)             # the cooperative engine (grid barriers)
        img0 = ctx.image_host(e, v, 0)
        # never-completing barrier, 4096 polls per CTA
        ctx.test_barrier_timeout(polls=4096, never_complete=True)
        echo = np.ascontiguousarray(e, np.complex64)
        img = np.full((M, 512), np.nan, np.float32)
        t0 = time.perf_counter()
        rc = lib.isar_image_host(ctx._h, echo.ctypes.data, v.ctypes.data, 0, img.ctypes.data)
        dt = time.perf_counter() - t0
        assert rc == ISAR_ECUDA
        assert "grid barrier timed out" in gb300.last_error()
        assert dt < 5.0                          # bounded: the limit, not a hang
        # the flag was reported once and cleared; normal operation again
        ctx.test_barrier_timeout(0, False)
        ctx.synchronize()
        img1 = ctx.image_host(e, v, 0)
    torch.cuda.synchronize()
    assert np.array_equal(img0, img1)
