"""Ingest parity: the drop-in dataParsing / dataExtracting (the reference's
.wbd reader, common.cu:750-1191, isar_imaging_export.cpp:48-119) against what
the reference's own ioOperation returns on the same files
(tests/golden/ingest_*.npz, made by tests/golden/make_golden.py from the
reference's sources compiled for the CPU).  The .wbd scenario
(tests/wbd.py) has three pitch blocks (45, 15 and 140 pulses), so the
turn-angle curve's block split, 20-pulse knots, pulse-by-pulse short block,
absolute-index knot lookup and block offsets are all exercised."""
import os
import subprocess

import numpy as np
import pytest

from oracle.ref_emu import read_dump
from tests.test_dropin import TMP, build_driver
from tests.wbd import write_ingest_scenario

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
# The turn angle is computed in float (sin, cos, acos of nearly parallel
# directions: ill-conditioned); one ulp of a libm result on another machine
# moves it by ~1e-4 relative.  Everything else is exact.
TA_RTOL = 2e-4


def _fixture(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def _scenario_dir(data_type):
    d = os.path.join(TMP, "ingest_%d" % data_type)
    os.makedirs(d, exist_ok=True)
    write_ingest_scenario(d, data_type=data_type)
    return d


@pytest.mark.parametrize("name", ["ingest_stretch", "ingest_ifds"])
def test_data_parsing_matches_the_reference(name):
    z = _fixture(name)
    dt = int(z["data_type"])
    exe = build_driver()
    d = _scenario_dir(dt)
    out = os.path.join(d, "parse.bin")
    r = subprocess.run([exe, "--parse-bin", d, "1", str(dt), out], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    fl, dn, ta = read_dump(out, (np.int32, np.float64, np.float32))
    assert (int(fl[0]), int(fl[1])) == (int(z["frame_len"]), int(z["frame_num"]))
    np.testing.assert_array_equal(dn, z["dataN"])          # range, velocity, azimuth, pitching
    assert np.isfinite(z["turnAngle"]).all()
    np.testing.assert_allclose(ta, z["turnAngle"], rtol=TA_RTOL, atol=1e-6)


@pytest.mark.gpu
def test_data_extracting_matches_the_reference(torch_cuda):
    z = _fixture("ingest_stretch")
    exe = build_driver()
    d = _scenario_dir(2)
    out = os.path.join(d, "extract.bin")
    window_len, window_head, stride = (int(v) for v in z["window"])
    r = subprocess.run([exe, "--extract-bin", d, "1", "2", str(window_len), str(window_head), str(stride), out],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    sn, dno, tao, dw = read_dump(out, (np.int32, np.float64, np.float32, np.float32))
    np.testing.assert_array_equal(sn, z["sn"])
    np.testing.assert_array_equal(dno, z["dataNOut"])
    np.testing.assert_allclose(tao, z["turnAngleOut"], rtol=TA_RTOL, atol=1e-6)
    np.testing.assert_array_equal(dw.view(np.complex64), z["dataW"])   # int16 samples as float
