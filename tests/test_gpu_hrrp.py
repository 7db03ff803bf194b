"""getHRRP (common.cu:541-580) on the GPU (isar_stage_hrrp) against the
reference's own getHRRP (golden fixtures hrrp_*.npz from its sources run on
the CPU) and the FP64 oracle, STRETCH and IFDS, out of place and in place."""
import glob
import os

import numpy as np
import pytest

import oracle
from tests.helpers import rel_l2

pytestmark = pytest.mark.gpu

HRRP_GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "hrrp_*.npz")))


def _run(torch, g, echo, data_type, inplace):
    M, N = echo.shape
    rp = g.radar(M, N, data_type=data_type)
    x = torch.from_numpy(np.ascontiguousarray(echo, np.complex64).view(np.float32).reshape(M, 2 * N).copy()).cuda()
    out = x if inplace else torch.full_like(x, np.nan)
    with g.Context(rp, stream=torch.cuda.current_stream().cuda_stream) as ctx:
        ctx.stage_hrrp(x, out)
        ctx.synchronize()
    o = out.cpu().numpy().reshape(M, N, 2)
    return o[..., 0] + 1j * o[..., 1]


@pytest.mark.parametrize("path", HRRP_GOLDEN, ids=[os.path.basename(p)[:-4] for p in HRRP_GOLDEN])
def test_hrrp_matches_reference_golden(torch_cuda, gb300, path):
    z = np.load(path)
    echo = oracle.iq_to_c64(z["iq"])
    dt = int(z["data_type"])
    # a context images >= 128 pulses: the fixture's rows repeated (rows are
    # independent)
    rep = 128 // echo.shape[0]
    want = oracle.hrrp(echo, dt)
    for inplace in (False, True):
        got = _run(torch_cuda, gb300, np.tile(echo, (rep, 1)), dt, inplace)
        for k in range(rep):
            blk = got[k * echo.shape[0]:(k + 1) * echo.shape[0]]
            assert rel_l2(blk, z["out"]) < 1e-5
            assert rel_l2(blk, want) < 1e-5


def test_hrrp_of_a_full_size_frame(torch_cuda, gb300):
    """1024 x 8192 STRETCH frame: every row equals the oracle's."""
    from tests.helpers import make_frame
    echo, _ = make_frame(1024, 8192, seed=5)
    got = _run(torch_cuda, gb300, echo, gb300.STRETCH, False)
    want = oracle.hrrp(echo, oracle.STRETCH)
    assert rel_l2(got, want) < 1e-5
