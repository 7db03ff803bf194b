"""The cluster-resident autofocus engine (one thread-block cluster per frame,
distributed shared memory) against the FP64 oracle, through the C ABI."""
import numpy as np
import pytest

import oracle
from tests.helpers import golden_echo, make_frame, rel_l2
from tests.test_gpu_parity import TOL_IMG, ctx_for, from_dev, to_dev

pytestmark = pytest.mark.gpu


def _cut(M, N, seed, full=False):
    e, _ = make_frame(M, N, seed=seed, full=full)
    rp = oracle.radar(M, N)
    y, _ = oracle.range_align(e, rp)
    _, cut, _ = oracle.center_cut(y, rp)
    return cut.astype(np.complex64)


def _cluster_or_skip(ctx, cl):
    mx = ctx.tuning().af_cluster_max
    if cl > mx:
        pytest.skip("cluster of %d CTAs not launchable here (max %d)" % (cl, mx))


@pytest.mark.parametrize("cl", [4, 8, 16])
@pytest.mark.parametrize("M,N,seed", [(128, 512, 1), (256, 1024, 2), (512, 2048, 3), (1024, 2048, 4)])
def test_cluster_fast_entropy_matches_oracle(torch_cuda, gb300, M, N, seed, cl):
    torch = torch_cuda
    cut = _cut(M, N, seed)
    want, tw = oracle.fast_entropy(cut)
    with ctx_for(gb300, torch, M, N) as ctx:
        _cluster_or_skip(ctx, cl)
        ctx.set_tuning(af_cluster=cl)
        dc = to_dev(torch, cut)
        ctx.stage_fast_entropy(dc, 120)
        got = from_dev(torch, dc).reshape(M, 512)
        tr = ctx.trace()
    assert tr["unit2_num"] == tw["unit2_num"]
    assert np.array_equal(tr["bins"], tw["bins"])
    assert tr["af_iterations"] == 120
    assert np.isfinite(tr["af_entropy"])
    assert rel_l2(got, want) < TOL_IMG


def test_cluster_many_bins_reload_path(torch_cuda, gb300):
    """M = 1024 with U = 256 bins: a cluster of 4 caches 16 of each CTA's 64
    bins and reloads the rest every iteration."""
    torch = torch_cuda
    M = 1024
    rng = np.random.default_rng(5)
    cut = (rng.standard_normal((M, 512)) + 1j * rng.standard_normal((M, 512))).astype(np.complex64) * 300
    # 280 constant-magnitude bright bins -> tgt_num 280, U = 256
    cut[:, 100:380] = (6000 * np.exp(2j * np.pi * rng.random((M, 280)))).astype(np.complex64)
    want, tw = oracle.fast_entropy(cut, iters=10)
    assert tw["unit2_num"] == 256
    with ctx_for(gb300, torch, M, 2048) as ctx:
        _cluster_or_skip(ctx, 4)
        ctx.set_tuning(af_cluster=4)
        dc = to_dev(torch, cut)
        ctx.stage_fast_entropy(dc, 10)
        got = from_dev(torch, dc).reshape(M, 512)
        tr = ctx.trace()
    assert tr["unit2_num"] == tw["unit2_num"]
    assert rel_l2(got, want) < TOL_IMG


def test_cluster_stop_criterion_equals_oracle_at_same_count(torch_cuda, gb300):
    torch = torch_cuda
    M, N = 256, 1024
    cut = _cut(M, N, 9)
    with ctx_for(gb300, torch, M, N) as ctx:
        _cluster_or_skip(ctx, 8)
        ctx.set_tuning(af_cluster=8, af_tol=1e-5, af_iters=120)
        dc = to_dev(torch, cut)
        ctx.stage_fast_entropy(dc, 120)
        got = from_dev(torch, dc).reshape(M, 512)
        tr = ctx.trace()
    k = tr["af_iterations"]
    assert 1 <= k < 120
    assert k % 4 == 0   # the criterion is checked every 4th iteration, before its update
    want, _ = oracle.fast_entropy(cut, iters=k)
    assert rel_l2(got, want) < TOL_IMG


def test_cluster_engine_whole_frame_matches_reference_golden(torch_cuda, gb300):
    import glob
    import os
    torch = torch_cuda
    for path in sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz"))):
        if os.path.basename(path).startswith(("pc_", "hrrp_", "ingest_")):   # stage fixtures, not frames
            continue
        z = np.load(path)
        M, N = int(z["M"]), int(z["N"])
        flags = (gb300.FLAG_HPC if bool(z["hpc"]) else 0) | (gb300.FLAG_MTRC if bool(z["mtrc"]) else 0)
        echo = golden_echo(z)
        rp = oracle.radar(M, N, B=float(z["B"]), fc=float(z["fc"]), Fs=float(z["Fs"]), Tp=float(z["Tp"]))
        _, tw = oracle.image(echo, z["velocity"], rp, hpc=bool(z["hpc"]), mtrc=bool(z["mtrc"]))
        with ctx_for(gb300, torch, M, N) as ctx:
            _cluster_or_skip(ctx, 8)
            ctx.set_tuning(af_cluster=8)
            ctx.set_ra_shifts(tw["ra_shift"])
            got = ctx.image_host(echo, z["velocity"], flags)
        assert rel_l2(got, z["img"]) < TOL_IMG, path
