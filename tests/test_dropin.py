"""Drop-in boundary: a C++ caller using only the reference's seven exports
(isar_imaging_export.h), in the call order of calling_dll.cpp, against
libisar_gb300.so on synthetic .wbd files."""
import os
import subprocess

import numpy as np
import pytest

import isar_imaging_cuda_gb300 as g
import oracle
from tests.helpers import CFG_FULL, full_omega
from tests.wbd import dropin_dir, write_wbd

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TMP = os.path.join(ROOT, "tests", "_tmp")
FS, TP = 128e6, 16e-6            # Tp = N / Fs in whole microseconds (the header stores us)


def build_driver():
    lib = g.lib_path()
    g.load()
    os.makedirs(TMP, exist_ok=True)
    exe = os.path.join(TMP, "dropin_main")
    src = os.path.join(ROOT, "tests", "dropin", "dropin_main.cpp")
    if not os.path.exists(exe) or os.path.getmtime(exe) < max(os.path.getmtime(src), os.path.getmtime(lib)):
        subprocess.check_call(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), src, "-o", exe,
                               lib, "-Wl,-rpath," + os.path.dirname(lib)])
    return exe


def frames(P, N, seed, full):
    cfg = dict(CFG_FULL) if full else {}
    if full:
        cfg["omega"] = full_omega(P)
    cfg.update(M=P, N=N, seed=seed, Fs=FS)
    return oracle.synth(cfg)


def test_data_parsing_decodes_the_navigation_header():
    exe = build_driver()
    P, N = 40, 512
    iq, vel = frames(P, N, seed=3, full=True)
    d = dropin_dir(TMP, "parse")
    az = np.linspace(10.0, 10.39, P)
    pit = np.full(P, 5.0)
    write_wbd(os.path.join(d, "syn_000004_1383_00_1101.wbd"), iq, vel, Fs=FS, Tp=TP, azimuth=az, pitching=pit,
              range_m=np.linspace(1000.0, 1003.9, P))
    out = subprocess.run([exe, "--parse", d, "1"], capture_output=True, text=True, check=True).stdout.split("\n")
    assert out[0] == "frame_len %d frame_num %d" % (4 * N + 256, P)
    rows = np.array([[float(v) for v in ln.split()] for ln in out[1:] if ln.strip()])
    assert rows.shape == (P, 6)
    np.testing.assert_allclose(rows[:, 1], np.round(np.linspace(1000.0, 1003.9, P) * 10) / 10, atol=1e-6)
    np.testing.assert_allclose(rows[:, 2], vel, atol=1e-6)                    # 0.1 m/s, signed
    np.testing.assert_allclose(rows[:, 3], az, atol=1e-4)
    np.testing.assert_allclose(rows[:, 4], pit, atol=1e-4)
    # turn angle: one block (pitching constant), 20-pulse steps interpolated,
    # monotone and close to the azimuth change times cos(pitching)
    ta = rows[:, 5]
    assert np.all(np.diff(ta) >= -1e-6)
    assert abs(ta[20] - (az[20] - az[0]) * np.cos(np.deg2rad(5.0))) < 2e-3


def test_data_parsing_rejects_an_empty_directory():
    exe = build_driver()
    d = dropin_dir(TMP, "empty")
    r = subprocess.run([exe, "--parse", d, "1"], capture_output=True, text=True)
    assert r.returncode == 4 and "No valid file" in r.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("full", [False, True])
def test_dropin_windows_match_the_c_abi(torch_cuda, full):
    exe = build_driver()
    M, N, stride, nwin = 256, 2048, 64, 3
    P = M + stride * (nwin - 1)
    iq, vel = frames(P, N, seed=77 + full, full=full)
    d = dropin_dir(TMP, "win%d" % full)
    for f in os.listdir(d):
        os.remove(os.path.join(d, f))
    write_wbd(os.path.join(d, "syn_000004_1383_00_1101.wbd"), iq, vel, Fs=FS, Tp=TP)
    prefix = os.path.join(d, "img_")
    r = subprocess.run([exe, d, "1", str(M), str(nwin), str(stride), str(int(full)), str(int(full)), prefix],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    echo = oracle.iq_to_c64(iq)
    flags = (g.FLAG_HPC | g.FLAG_MTRC) if full else 0
    with g.Context(g.radar(M, N, Fs=FS, Tp=TP)) as ctx:
        for w in range(nwin):
            got = np.loadtxt(prefix + "%d.txt" % w).reshape(M, 512)
            want = ctx.image_host(echo[w * stride:w * stride + M], vel[w * stride:w * stride + M], flags)
            # writeFileFLT keeps 5 decimals
            assert np.max(np.abs(got - want)) <= 6e-6 + 1e-6 * np.max(np.abs(want))


@pytest.mark.gpu
def test_dropin_ifds_windows_match_the_c_abi(torch_cuda):
    """IFDS data through the seven exports: dataExtracting pulse-compresses
    the new pulses of every window (isar_pulse_compress, one launch) with the
    reference's velocity index dataNOut[echo_num + dataWFileSn[i]], then
    isarMainSingle images them; equal to the C ABI path on the same pulses."""
    from tests.helpers import make_ifds_pulses
    torch = torch_cuda
    exe = build_driver()
    M, stride, nwin = 128, 32, 3
    P = M + stride * (nwin - 1)
    iq_len, fs, tp, B, fc = 5000, 200e6, 10e-6, 100e6, 10e9
    ad, _ = make_ifds_pulses(P, iq_len, fs, tp, B, seed=91, n_scat=4)
    nav_vel = np.linspace(-50.0, 50.0, P)   # navigation velocity per frame, m/s
    d = dropin_dir(TMP, "ifds")
    for f in os.listdir(d):
        os.remove(os.path.join(d, f))
    # the IFDS header stores twice the sampling rate (getSystemParas halves it)
    write_wbd(os.path.join(d, "syn_000004_1383_01_1101.wbd"), ad.reshape(P, iq_len, 2), nav_vel, fc=fc, B=B,
              Tp=tp, Fs=2 * fs)
    prefix = os.path.join(d, "img_")
    r = subprocess.run([exe, d, "1", str(M), str(nwin), str(stride), "0", "1", prefix, "1"], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    rp = g.radar(M, 4096, B=B, fc=fc, Fs=fs, Tp=tp, data_type=g.IFDS)
    # navigation values as dataParsing decodes them (0.1 m/s, 360/2^24 degrees)
    dec_vel = np.round(nav_vel * 10) * 0.1
    dec_az = np.round(np.linspace(10.0, 10.5, P) * (1 << 24) / 360.0) * (360.0 / (1 << 24))
    dec_pit = np.round(5.0 * (1 << 24) / 360.0) * (360.0 / (1 << 24))
    used = np.zeros(P)   # velocity each pulse was compressed with
    with g.Context(rp, stream=torch.cuda.current_stream().cuda_stream) as ctx:
        for w in range(nwin):
            head = w * stride
            sn = head + np.arange(M)
            # dataNOut = [range, velocity, azimuth, pitching] of the window's
            # pulses; the reference reads pulse i's velocity at M + sn_i, for
            # the new pulses only (the overlap keeps the previous window's rows)
            dn = np.concatenate([np.full(M, 1000.0), dec_vel[sn], dec_az[sn], np.full(M, dec_pit)])
            new = sn[(M - stride if w else 0):]
            used[new] = dn[M + new]
            vel = used[sn]
            echo = torch.zeros((M, 4096, 2), dtype=torch.float32, device="cuda")
            ctx.pulse_compress(torch.from_numpy(ad[sn].copy()).cuda(), iq_len,
                               torch.from_numpy(vel.copy()).cuda(), echo)
            img = torch.zeros((M, 512), dtype=torch.float32, device="cuda")
            ctx.image_device(echo, None, img, g.FLAG_MTRC)
            ctx.synchronize()
            want = img.cpu().numpy()
            got = np.loadtxt(prefix + "%d.txt" % w).reshape(M, 512)
            assert np.max(np.abs(got - want)) <= 6e-6 + 1e-6 * np.max(np.abs(want)), w
