"""Batched imaging (one CUDA graph over frames of uneven size) and the
autotuner, through the C ABI: equal to single-frame imaging with the same
launch parameters, and to the FP64 oracle."""
import numpy as np
import pytest

import oracle
from tests.helpers import make_frame, rel_l2
from tests.test_gpu_parity import TOL_IMG

pytestmark = pytest.mark.gpu

# (M, N, full, seed): uneven pulse and range-cell counts, plain and
# five-stage frames mixed, two frames sharing each of two shapes
FRAMES = [(128, 512, False, 41), (256, 1024, False, 42), (128, 1024, False, 43), (256, 1024, False, 44),
          (128, 512, False, 45), (256, 2048, True, 46)]


def _frames_on_device(torch, g):
    out = []
    for M, N, full, seed in FRAMES:
        e, v = make_frame(M, N, seed=seed, full=full)
        de = torch.from_numpy(np.ascontiguousarray(e, np.complex64).view(np.float32).copy()).cuda()
        dv = torch.from_numpy(np.ascontiguousarray(v, np.float64).copy()).cuda()
        img = torch.full((M, 512), np.nan, dtype=torch.float32, device="cuda")
        flags = (g.FLAG_HPC | g.FLAG_MTRC) if full else 0
        out.append(dict(M=M, N=N, full=full, e=e, v=v, de=de, dv=dv, img=img, flags=flags, rp=g.radar(M, N)))
    return out


def _batch_list(g, fr):
    return g.Batch.frames((f["rp"], f["de"], f["dv"] if f["full"] else None, f["flags"], f["img"]) for f in fr)


def test_batch_equals_single_frame_and_oracle(torch_cuda, gb300):
    torch = torch_cuda
    fr = _frames_on_device(torch, gb300)
    with gb300.Batch(lanes=2) as b:
        lst = _batch_list(gb300, fr)
        b.run(lst)
        b.synchronize()
        got = [f["img"].cpu().numpy().copy() for f in fr]
        # a replay of the cached graph gives the same images
        for f in fr:
            f["img"].fill_(np.nan)
        b.run(lst)
        b.synchronize()
        for f, g0 in zip(fr, got):
            assert np.array_equal(f["img"].cpu().numpy(), g0)
        tunings = {(f["M"], f["N"]): b.tuning(f["rp"]) for f in fr}
    for f, img in zip(fr, got):
        t = tunings[(f["M"], f["N"])]
        assert t.af_cluster > 0
        with gb300.Context(f["rp"], stream=torch.cuda.current_stream().cuda_stream) as ctx:
            ctx.set_tuning(**{k: getattr(t, k) for k in ("ra_rows_each_level", "ra_pair_min", "ra_rows_per_cta", "ra_rows_final",
                                                         "af_cluster", "af_tol", "af_iters")})
            single = ctx.image_host(f["e"], f["v"], f["flags"])
        assert rel_l2(img, single) <= 1e-6, (f["M"], f["N"])
        want, _ = oracle.image(f["e"], f["v"], oracle.radar(f["M"], f["N"]), hpc=f["full"], mtrc=f["full"])
        assert rel_l2(img, want) < TOL_IMG, (f["M"], f["N"])


# the benchmark's frame size and its half, five-stage, beside a plain frame
LARGE = [(1024, 8192, True, 51), (512, 4096, True, 52), (256, 4096, False, 53), (1024, 8192, True, 54)]


def test_batch_of_large_uneven_frames_equals_single_frame_and_oracle(torch_cuda, gb300):
    torch = torch_cuda
    fr = []
    for M, N, full, seed in LARGE:
        e, v = make_frame(M, N, seed=seed, full=full)
        fr.append(dict(M=M, N=N, full=full, e=e, v=v, rp=gb300.radar(M, N),
                       de=torch.from_numpy(np.ascontiguousarray(e, np.complex64).view(np.float32).copy()).cuda(),
                       dv=torch.from_numpy(np.ascontiguousarray(v, np.float64).copy()).cuda(),
                       img=torch.full((M, 512), np.nan, dtype=torch.float32, device="cuda"),
                       flags=(gb300.FLAG_HPC | gb300.FLAG_MTRC) if full else 0))
    with gb300.Batch(lanes=2) as b:
        b.run(_batch_list(gb300, fr))
        b.synchronize()
        tunings = {(f["M"], f["N"]): b.tuning(f["rp"]) for f in fr}
    for f in fr:
        img = f["img"].cpu().numpy()
        t = tunings[(f["M"], f["N"])]
        with gb300.Context(f["rp"], stream=torch.cuda.current_stream().cuda_stream) as ctx:
            ctx.set_tuning(**{k: getattr(t, k) for k in ("ra_rows_each_level", "ra_pair_min", "ra_rows_per_cta",
                                                         "ra_rows_final", "af_cluster", "af_tol", "af_iters")})
            single = ctx.image_host(f["e"], f["v"], f["flags"])
        assert rel_l2(img, single) <= 1e-6, (f["M"], f["N"])
        want, _ = oracle.image(f["e"], f["v"], oracle.radar(f["M"], f["N"]), hpc=f["full"], mtrc=f["full"])
        assert rel_l2(img, want) < TOL_IMG, (f["M"], f["N"])
        assert abs(oracle.entropy(img) - oracle.entropy(want)) < 1e-4


def test_batch_autotune_keeps_results(torch_cuda, gb300):
    torch = torch_cuda
    fr = _frames_on_device(torch, gb300)[:4]
    with gb300.Batch() as b:
        lst = _batch_list(gb300, fr)
        ms = b.autotune(lst)
        assert 0.0 < ms < 1e4
        assert b.lanes() in (1, 2, 4, 8, 16, 32, 64, 128)
        b.run(lst)
        b.synchronize()
        for f in fr:
            t = b.tuning(f["rp"])
            assert t.af_cluster in (4, 8, 16) and t.ra_pair_min >= 1
    for f in fr:
        want, _ = oracle.image(f["e"], f["v"], oracle.radar(f["M"], f["N"]), hpc=f["full"], mtrc=f["full"])
        assert rel_l2(f["img"].cpu().numpy(), want) < TOL_IMG


def test_context_autotune_cooperative_or_cluster(torch_cuda, gb300):
    torch = torch_cuda
    M, N = 256, 1024
    e, v = make_frame(M, N, seed=77)
    de = torch.from_numpy(np.ascontiguousarray(e, np.complex64).view(np.float32).copy()).cuda()
    want, _ = oracle.image(e, v, oracle.radar(M, N))
    with gb300.Context(gb300.radar(M, N), stream=torch.cuda.current_stream().cuda_stream) as ctx:
        t = ctx.autotune(de, None, 0, engines=3)
        assert t.af_cluster in (0, 4, 8, 16)
        got = ctx.image_host(e, v, 0)
    assert rel_l2(got, want) < TOL_IMG


def test_misaligned_echo_is_rejected_before_any_launch(torch_cuda, gb300):
    """Rows are staged into shared memory by 16-byte bulk copies: an echo
    buffer that is only 8-byte aligned is refused on the host (EINVAL)."""
    torch = torch_cuda
    M, N = 128, 512
    base = torch.zeros(2 * M * N + 2, dtype=torch.float32, device="cuda")
    odd = base[2:]   # 8 bytes past a 16-byte boundary
    assert odd.data_ptr() % 16 == 8
    vel = torch.zeros(M, dtype=torch.float64, device="cuda")
    img = torch.zeros((M, 512), dtype=torch.float32, device="cuda")
    rp = gb300.radar(M, N)
    with gb300.Context(rp, stream=torch.cuda.current_stream().cuda_stream) as ctx:
        with pytest.raises(gb300.IsarError, match="16-byte aligned"):
            ctx.stage_range_align(odd, vel, 0)
        with pytest.raises(gb300.IsarError, match="16-byte aligned"):
            ctx.image_device(odd, vel, img, 0)
    with gb300.Batch(lanes=1) as b:
        with pytest.raises(gb300.IsarError, match="16-byte aligned"):
            b.run(gb300.Batch.frames([(rp, odd, None, 0, img)]))


def test_iq16_conversion_matches_the_host_cast(torch_cuda, gb300):
    """isar_iq16_to_c64: the int16 -> float cast of getSignalData
    (common.cu:1096-1098), done on the device; odd sample counts included."""
    torch = torch_cuda
    rng = np.random.default_rng(3)
    for n in (1, 2, 7, 1000, 1 << 20):
        iq = rng.integers(-32768, 32767, size=(n, 2), dtype=np.int16)
        d_iq = torch.from_numpy(iq).cuda()
        d_out = torch.full((n, 2), np.nan, dtype=torch.float32, device="cuda")
        gb300.iq16_to_c64(d_iq, d_out, torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        assert np.array_equal(d_out.cpu().numpy(), iq.astype(np.float32))


@pytest.mark.parametrize("M,N,full,ifds", [(256, 1024, True, False), (128, 2048, False, False),
                                           (128, 4096, False, True)])
def test_iq16_echoes_image_like_complex64_echoes(torch_cuda, gb300, M, N, full, ifds):
    """ISAR_FLAG_IQ16: the int16 samples read directly by range alignment (or
    converted for the IFDS pre-step) give bit-identical images to the same
    samples as complex64, single frame and batched."""
    torch = torch_cuda
    echo, vel = make_frame(M, N, seed=61, full=full)
    iq = np.stack([echo.real, echo.imag], -1).astype(np.int16)   # the frames are int16-quantised
    assert np.array_equal(iq.astype(np.float32), np.stack([echo.real, echo.imag], -1))
    d_f = torch.from_numpy(np.ascontiguousarray(iq.astype(np.float32)).reshape(M, 2 * N)).cuda()
    d_q = torch.from_numpy(np.ascontiguousarray(iq).reshape(M, 2 * N)).cuda()
    d_v = torch.from_numpy(np.ascontiguousarray(vel, np.float64)).cuda()
    flags = (gb300.FLAG_HPC | gb300.FLAG_MTRC) if full else 0
    rp = gb300.radar(M, N, data_type=gb300.IFDS if ifds else gb300.STRETCH)
    out = {}
    with gb300.Context(rp, stream=torch.cuda.current_stream().cuda_stream) as ctx:
        for name, x, f in (("f32", d_f, flags), ("i16", d_q, flags | gb300.FLAG_IQ16)):
            img = torch.zeros((M, 512), dtype=torch.float32, device="cuda")
            ctx.image_device(x, d_v, img, f)
            ctx.image_device(x, d_v, img, f)   # second call: graph replay
            ctx.synchronize()
            out[name] = img.cpu().numpy()
    assert np.array_equal(out["f32"], out["i16"])
    if not ifds:
        imgs = [torch.zeros((M, 512), dtype=torch.float32, device="cuda") for _ in range(2)]
        with gb300.Batch(lanes=2) as b:
            b.run(gb300.Batch.frames([(rp, d_q, d_v, flags | gb300.FLAG_IQ16, imgs[0]),
                                      (rp, d_f, d_v, flags, imgs[1])]))
            b.synchronize()
        assert np.array_equal(imgs[0].cpu().numpy(), imgs[1].cpu().numpy())
