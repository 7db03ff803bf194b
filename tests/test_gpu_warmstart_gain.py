"""What the trained warm-start network gains over the method without it, on
held-out synthetic frames (seeds disjoint from the training seeds).

Each frame runs the judged warm start: the autofocus from the network's start
until the entropy stop criterion (the learned leg), the autofocus from the
Doppler-tracking start until the same criterion (the plain leg, the method
without the network), and the lower final entropy of the selected bins is
kept.  From one run per frame the test reads both legs' iterations and final
entropies, and compares the judged image with the reference's fixed 120
iterations.  The measured gain is printed."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-6   # stop criterion of both legs


def test_trained_warm_start_gain_and_judge(torch_cuda, gb300):
    from isar_imaging_cuda_gb300 import warmstart as W
    path = gb300.WARMSTART_WEIGHTS
    assert os.path.exists(path), path
    params = np.load(path)
    rows = W.evaluate_autofocus(torch_cuda, params, "poly", 96, tol=TOL)
    s = W.summarize(rows)
    print("warm-start gain:", json.dumps(s))
    # the judge: the kept result is never the worse leg
    for r in rows:
        e_plain, e_learned = r["judged"]["legs_entropy"]
        kept = e_learned if r["judged"]["ws_used"] else e_plain
        assert kept <= min(e_plain, e_learned)
        assert r["judged"]["iters"] == sum(r["judged"]["legs_iters"])
    # the network's gain: its leg reaches the stop criterion in fewer
    # iterations than the plain leg, and is kept on part of the frames
    assert s["iters_learned_leg"] < s["iters_plain_leg"], s
    assert s["learned_kept_frac"] > 0.0, s
