"""The oracle against golden vectors produced by the reference's own code
(tests/golden/make_golden.py: the reference sources compiled for the CPU by
oracle/ref_emu and driven through imagingMemInit + isarMainSingle)."""
import glob
import os

import numpy as np
import pytest

import oracle
from tests.helpers import golden_echo, rel_l2

GOLDEN = sorted(p for p in glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz"))
                if not os.path.basename(p).startswith(("pc_", "hrrp_", "ingest_")))
PC_GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "pc_*.npz")))
HRRP_GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "hrrp_*.npz")))


def load(path):
    z = np.load(path)
    M, N = int(z["M"]), int(z["N"])
    rp = oracle.radar(M, N, B=float(z["B"]), fc=float(z["fc"]), Fs=float(z["Fs"]), Tp=float(z["Tp"]))
    return z, M, N, rp


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_oracle_matches_reference_golden(path):
    z, M, N, rp = load(path)
    echo = golden_echo(z)
    hpc, mtrc = bool(z["hpc"]), bool(z["mtrc"])
    img, tr = oracle.image(echo, z["velocity"], rp, hpc=hpc, mtrc=mtrc)
    # whole frame: image within the acceptance bar, same entropy
    assert rel_l2(img, z["img"]) < 1e-4
    assert abs(oracle.entropy(img) - oracle.entropy(z["img"].astype(np.float64))) < 1e-4
    # stage checkpoint (fixtures that store it): centring + cut (pins the
    # integer centring shift and the cut offset: a one-cell difference would
    # give rel L2 ~ 1)
    if "cut" not in z:
        return
    x = oracle.hpc(echo, z["velocity"], rp) if hpc else echo
    y, _ = oracle.range_align(x, rp)
    _, cut, _ = oracle.center_cut(y, rp)
    assert rel_l2(cut, z["cut"]) < 1e-4


def test_goldens_present():
    assert len(GOLDEN) >= 2
    assert len(PC_GOLDEN) >= 3
    assert len(HRRP_GOLDEN) >= 2


@pytest.mark.parametrize("path", HRRP_GOLDEN, ids=[os.path.basename(p)[:-4] for p in HRRP_GOLDEN])
def test_oracle_hrrp_matches_reference_golden(path):
    """getHRRP (common.cu:541-580), STRETCH and IFDS: the oracle against the
    reference's own getHRRP run on the CPU."""
    z = np.load(path)
    got = oracle.hrrp(oracle.iq_to_c64(z["iq"]), int(z["data_type"]))
    assert rel_l2(got, z["out"]) < 1e-6


def pc_radar(z):
    return oracle.Radar(0, 4096, int(float(z["B"])), int(float(z["fc"])), float(z["Tp"]), int(float(z["Fs"])))


@pytest.mark.parametrize("path", PC_GOLDEN, ids=[os.path.basename(p)[:-4] for p in PC_GOLDEN])
def test_oracle_pulse_compression_matches_reference_golden(path):
    """IFDS pulse compression (common.cu:583-604, 635-746): the oracle against
    the reference's pulseCompression class run on the CPU.  The cut offset
    is pinned exactly (a one-cell difference gives rel L2 ~ 1)."""
    z = np.load(path)
    out, offs = oracle.pulse_compress(z["ad"], z["velocity"], pc_radar(z))
    assert out.shape == z["out"].shape
    for p in range(out.shape[0]):
        assert rel_l2(out[p], z["out"][p]) < 1e-5, p
    # the compressed pulses carry their targets: a clear peak in the cut
    pk = np.abs(out).max(axis=1) / np.median(np.abs(out), axis=1)
    assert (pk > 20).all()


def test_launch_rewrite_of_the_emulation_recipe():
    from oracle import ref_emu
    src = "\tifftshiftRows << <dim3(((n / 2) + b.x - 1) / b.x, m), b >> > (d, n);\n\tx = a >> 1;"
    out = ref_emu.transform(src)
    assert "EMU_LAUNCH(ifftshiftRows, dim3(((n / 2) + b.x - 1) / b.x, m), b )(d, n);" in out
    assert "x = a >> 1;" in out
