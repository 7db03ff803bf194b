"""What the trained warm-start network gains over the method without it, on
held-out synthetic frames (seeds disjoint from the training seeds): mean
autofocus iterations to the same entropy stop criterion, and final image
entropy against the reference's fixed 120 iterations.  The control arm is a
network that predicts no correction (the Doppler-tracking start with pulse 0
kept), so the gain measured is the trained network's own.

Measured gain on these workloads is small (a few percent fewer iterations):
the Doppler-tracking increments are already within ~0.01 rad of the
autofocus fixed point, and what the autofocus spends its iterations on is the
low-frequency accumulation of those small errors.  The test therefore checks
that the trained start is kept on part of the frames, costs no iterations and
no entropy against the control, and prints the measured numbers."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_trained_warm_start_against_zero_correction_control(torch_cuda, gb300):
    from isar_imaging_cuda_gb300 import warmstart as W
    path = gb300.WARMSTART_WEIGHTS
    assert os.path.exists(path), path
    params = np.load(path)
    rows = W.evaluate_autofocus(torch_cuda, params, "poly", 96, tol=1e-6)
    s = W.summarize(rows)
    print("warm-start gain:", json.dumps(s))
    assert s["learned"]["ws_used_frac"] > 0.0
    assert s["learned"]["iters_mean"] <= s["doppler1"]["iters_mean"] + 1.0, s
    # Different starts can settle in different local minima, so single frames
    # move by up to ~1e-2 either way; the typical frame must not get worse.
    e120 = np.array([r["ref120"]["entropy"] for r in rows])
    med = {m: float(np.median(np.array([r[m]["entropy"] for r in rows]) - e120)) for m in ("doppler1", "learned")}
    print("median entropy change against 120 iterations:", med)
    assert med["learned"] <= med["doppler1"] + 1e-4, med
