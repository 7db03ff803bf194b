"""The CPU restatement of the warm-start network (oracle/wsnet.py): its
backward pass against central finite differences (float64, no bf16
rounding), and the parameter layout against the library's count."""
import numpy as np
import pytest

from oracle import wsnet


def test_param_count_matches_library():
    import isar_imaging_cuda_gb300 as g
    assert wsnet.n_params() == g.load().isar_wsnet_param_count()


def test_bf16_rounding_ties_to_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 1e-30], np.float32)
    y = wsnet.bf16(x)
    assert y[0] == 1.0 and y[1] == 1.0 and y[2] == 1.0 + 2 ** -6 and y[3] == -2.5


@pytest.mark.parametrize("seed", [0, 1])
def test_backward_matches_finite_differences(seed):
    rng = np.random.default_rng(seed)
    F, M = 2, 16
    p = wsnet.init_params(seed, out_scale=0.3).astype(np.float64)
    x0 = rng.standard_normal((F, M, wsnet.CH)) * 0.5
    target = rng.uniform(-1.0, 1.0, (F, M))
    _, g = wsnet.loss_grad(p, x0, target, emulate=False)
    # parameters from every layer: weights and biases
    idx = []
    o = 0
    for r, c in wsnet.layer_shapes():
        idx += list(rng.choice(r * c, 3, replace=False) + o)
        o += r * c
        idx += list(rng.choice(r, 1) + o)
        o += r
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        lp, _ = wsnet.loss_grad(pp, x0, target, emulate=False)
        lm, _ = wsnet.loss_grad(pm, x0, target, emulate=False)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(fd), (i, fd, g[i])
