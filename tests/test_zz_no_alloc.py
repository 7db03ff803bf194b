"""isar_center_cut_noalloc (static device scratch, no allocation) against the
context entry point isar_stage_center_cut, called through the C ABI.

The file name sorts last so that the GPU test also runs after every other
test in one session; it passes on its own as well."""
import ctypes as C

import numpy as np
import pytest

import oracle
from tests.helpers import make_frame

# Same kernels on the same profiles: the cut must be bit-identical.
TOL_CUT = 0.0


def _profiles_on_device(torch, g, M, N, seed):
    """Range profiles made by the context path (range alignment stage)."""
    e, _ = make_frame(M, N, seed=seed)
    d = torch.from_numpy(np.ascontiguousarray(e, np.complex64).view(np.float32).copy()).cuda()
    with g.Context(g.radar(M, N), stream=torch.cuda.current_stream().cuda_stream) as ctx:
        ctx.stage_range_align(d)
        ref = torch.empty((M, 1024), dtype=torch.float32, device="cuda")
        ctx.stage_center_cut(d, ref)
        ctx.synchronize()
    return d, ref


def test_noalloc_rejects_oversized_range_num_without_gpu_work(gb300):
    lib = gb300.load()
    # Argument checks come before any CUDA call, so this runs without a GPU.
    ISAR_EINVAL = -1
    rc = lib.isar_center_cut_noalloc(C.c_void_p(16), 256, 16384, C.c_void_p(16), None)
    assert rc == ISAR_EINVAL
    assert "8192" in gb300.last_error()
    assert lib.isar_center_cut_noalloc(None, 256, 1024, C.c_void_p(16), None) == ISAR_EINVAL
    # pulse counts outside those of isar_create (powers of two in [128, 1024])
    for m in (300, 64, 2048):
        assert lib.isar_center_cut_noalloc(C.c_void_p(16), m, 1024, C.c_void_p(16), None) == ISAR_EINVAL
        assert "echo_num" in gb300.last_error()


@pytest.mark.gpu
def test_noalloc_center_cut_matches_context_path_two_calls_in_a_row(torch_cuda, gb300):
    torch = torch_cuda
    lib = gb300.load()
    stream = torch.cuda.current_stream().cuda_stream
    torch.cuda.synchronize()
    torch_before = torch.cuda.memory_allocated()
    # the set-up call (all arguments NULL/0) takes the scratch's address; it
    # makes no allocation of its own
    assert lib.isar_center_cut_noalloc(None, 0, 0, None, None) == 0, gb300.last_error()
    assert torch.cuda.memory_allocated() == torch_before

    cases = [(256, 8192, 11), (128, 1024, 12)]
    inputs = [_profiles_on_device(torch, gb300, M, N, seed) for M, N, seed in cases]
    outs = [torch.full((M, 1024), np.nan, dtype=torch.float32, device="cuda") for M, _, _ in cases]
    torch.cuda.synchronize()
    torch_before = torch.cuda.memory_allocated()
    free_before, _ = torch.cuda.mem_get_info()
    n0 = gb300.launch_count()
    for (M, N, _), (d_y, _), d_cut in zip(cases, inputs, outs):
        rc = lib.isar_center_cut_noalloc(d_y.data_ptr(), M, N, d_cut.data_ptr(), stream)
        assert rc == 0, gb300.last_error()
    torch.cuda.synchronize()
    assert gb300.launch_count() > n0
    # the two calls allocated nothing: neither through torch nor on the device
    assert torch.cuda.memory_allocated() == torch_before
    assert torch.cuda.mem_get_info()[0] == free_before
    for (M, N, _), (_, ref), d_cut in zip(cases, inputs, outs):
        got = d_cut.cpu().numpy().view(np.complex64)
        want = ref.cpu().numpy().view(np.complex64)
        assert np.isfinite(got).all()
        err = float(np.linalg.norm(got - want) / np.linalg.norm(want))
        assert err <= TOL_CUT, (M, N, err)

    # The oracle's decisions on the same profiles agree as well (same cut).
    M, N, _ = cases[1]
    y = inputs[1][0].cpu().numpy().view(np.complex64).reshape(M, N)
    _, cut_want, _ = oracle.center_cut(y.astype(np.complex128), oracle.radar(M, N))
    got = outs[1].cpu().numpy().view(np.complex64).reshape(M, 512)
    assert float(np.linalg.norm(got - cut_want) / np.linalg.norm(cut_want)) < 1e-5
