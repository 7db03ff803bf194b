"""What the trained warm-start network gains over the method without it, on
held-out synthetic frames (seeds disjoint from the training seeds): mean
autofocus iterations to the same entropy stop criterion, and final image
entropy against the reference's fixed 120 iterations.  The control arm is a
network that predicts no correction (the Doppler-tracking start with pulse 0
kept), so the gain measured is the trained network's own."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_trained_warm_start_needs_fewer_iterations(torch_cuda, gb300):
    from isar_imaging_cuda_gb300 import warmstart as W
    path = gb300.WARMSTART_WEIGHTS
    assert os.path.exists(path), path
    params = np.load(path)
    rows = W.evaluate_autofocus(torch_cuda, params, "poly", 48, tol=1e-6)
    s = W.summarize(rows)
    assert s["learned"]["ws_used_frac"] > 0.0
    assert s["learned"]["iters_mean"] < s["doppler1"]["iters_mean"], s
    # same stop criterion, final entropy no worse on average than the control
    assert s["learned"]["dE_vs_ref120_mean"] <= s["doppler1"]["dE_vs_ref120_mean"] + 1e-4, s
