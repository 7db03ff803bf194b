"""Training and evaluation of the learned autofocus warm start.

Data: frames generated on the GPU by isar_synth_device with known injected
per-pulse phase errors phi_m, pushed through the imaging pipeline's own
range alignment, centring, cut and bin selection (isar_frame_features).  The
label of pulse m is the residual of the Doppler-tracking increment,
r_m = wrap(psi_m - (phi_{m+1} - phi_m)).  Training runs on the GPU through the
network's own forward/backward/Adam kernels (isar_wsnet_*).

Workloads:
  * "poly": 256 x 1024 frames, phase error = random polynomial (order 2..6,
    coefficients N(0, pi)) + uniform +-0.5 rad, the plain-pipeline scene
    (50 scatterers in 20 m x 20 m, 0.02 rad/s, drift 0.3 cell, SNR 10 dB);
  * "full": 1024 x 8192 five-stage frames (200 scatterers in 40 m x 40 m, 4
    degrees, 3000 m/s + 50 m/s^2, quadratic + uniform phase error, SNR 5 dB).

    python -m isar_imaging_cuda_gb300.warmstart --out isar_imaging_cuda_gb300/weights/warmstart.npy

The committed weights came from that command (200k "poly" + 2k "full"
frames, 40 epochs; on one GB300: 358 s of data generation, 111 s of
training; held-out loss 2.77e-5 against 3.81e-5 for no correction).
"""
import argparse
import json
import math
import time

import numpy as np

from . import (FLAG_HPC, FLAG_MTRC, Context, WSNet, radar, synth_device, synth_params)

TRAIN_SEED0 = 5_000_000      # training seeds; evaluation uses EVAL_SEED0 + i
EVAL_SEED0 = 9_000_000


def workload(kind):
    if kind == "poly":
        return dict(M=256, N=1024, full=False, flags=0)
    if kind == "full":
        return dict(M=1024, N=8192, full=True, flags=FLAG_HPC | FLAG_MTRC)
    raise ValueError(kind)


def frame_params(kind, seed, rng):
    w = workload(kind)
    if kind == "poly":
        return synth_params(w["M"], w["N"], seed=seed, phase_uniform=0.5,
                            phase_poly_order=int(rng.integers(2, 7)), phase_poly_sigma=math.pi)
    return synth_params(w["M"], w["N"], seed=seed, full=True)


def make_dataset(torch, kind, n, seed0, label="teacher", cluster=16):
    """Features X [n][M][64] bf16 and labels R [n][M] fp32 (device).

    label "teacher": r_m = wrap(psi_m - (t_{m+1} - t_m)) with exp(-j t) the
    phase the reference autofocus (120 iterations, Doppler start) converges
    to on this frame, i.e. the network learns to start at that fixed point;
    label "injected": t = the generator's injected phase (error + drift
    carrier phase).  All work is ordered on one stream."""
    w = workload(kind)
    M, N = w["M"], w["N"]
    s = torch.cuda.Stream()
    X = torch.empty((n, M, 64), dtype=torch.bfloat16, device="cuda")
    P = torch.empty((n, M), dtype=torch.float32, device="cuda")
    theta = np.zeros((n, M), np.float64)
    x = torch.empty((M, 2 * N), dtype=torch.float32, device="cuda")
    v = torch.empty(M, dtype=torch.float64, device="cuda")
    img = torch.empty((M, 512), dtype=torch.float32, device="cuda")
    rng = np.random.default_rng(seed0)
    with torch.cuda.stream(s), Context(radar(M, N), stream=s.cuda_stream) as ctx:
        if label == "teacher":
            ctx.set_tuning(af_cluster=min(cluster, ctx.tuning().af_cluster_max), af_tol=0.0, af_iters=120)
        for i in range(n):
            _, pe = synth_device(frame_params(kind, seed0 + i, rng), x, v, s.cuda_stream, phase_err=True)
            ctx.features(x, v, w["flags"], X[i], P[i])
            if label == "teacher":
                ctx.image_device(x, v, img, w["flags"])
                theta[i] = -np.angle(ctx.trace()["phase"].astype(np.complex128))
            else:
                theta[i] = pe
        s.synchronize()
    psi = P.cpu().numpy().astype(np.float64)
    r = psi[:, :-1] - np.diff(theta, axis=1)
    r = np.angle(np.exp(1j * r))
    R = np.zeros((n, M), np.float32)
    R[:, :-1] = r
    return X, torch.from_numpy(R).cuda(), psi


LAYERS = [(64, 320)] * 6 + [(64, 64), (2, 64)]   # (rows, cols) of each weight, canonical order


def init_params(seed=0, out_scale=0.01):
    """He-normal hidden weights, zero hidden biases; a small last layer with
    bias (1, 0) so that the untrained network predicts r = 0 (the
    Doppler-tracking start)."""
    rng = np.random.default_rng(seed)
    parts = []
    for li, (r, c) in enumerate(LAYERS):
        last = li == len(LAYERS) - 1
        parts.append((rng.standard_normal((r, c)) * (out_scale if last else math.sqrt(2.0 / c))).ravel())
        parts.append(np.array([1.0, 0.0]) if last else np.zeros(r))
    return np.concatenate(parts).astype(np.float32)


def train(torch, sets, epochs=20, rows=32768, lr=2e-3, seed=0, log=print):
    """sets: list of (X, R) per workload.  Returns the parameters (numpy)."""
    net = WSNet(rows, training=True)
    net.set_params(init_params(seed))
    rng = np.random.default_rng(seed)
    batches = []
    for si, (X, R) in enumerate(sets):
        n, M = X.shape[0], X.shape[1]
        fb = max(1, rows // M)
        batches += [(si, j, min(j + fb, n)) for j in range(0, n, fb)]
    total = epochs * len(batches)
    step = 0
    hist = []
    t0 = time.time()
    for ep in range(epochs):
        order = rng.permutation(len(batches))
        perms = [torch.randperm(X.shape[0], device="cuda") for X, _ in sets]
        el = []
        for bi in order:
            si, j0, j1 = batches[bi]
            X, R = sets[si]
            idx = perms[si][j0:j1]
            xb = X[idx].contiguous()
            rb = R[idx].contiguous()
            f, M = xb.shape[0], xb.shape[1]
            net.forward(xb, f, M)
            el.append(net.backward(rb, f, M))
            step += 1
            net.adam(lr * max(0.5 * (1.0 + math.cos(math.pi * step / total)), 0.02))
        hist.append(float(np.mean(el)))
        log("epoch %d loss %.5f (%.1f s)" % (ep, hist[-1], time.time() - t0))
    p = net.params()
    net.close()
    return p, hist


def eval_loss(torch, params, X, R):
    """Mean loss of the network and of the untrained start (r_hat = 0)."""
    n, M = X.shape[0], X.shape[1]
    net = WSNet(n * M, training=True)
    net.set_params(params)
    net.forward(X, n, M)
    l_net = net.backward(R, n, M)
    net.close()
    r = R.cpu().numpy()[:, :-1].astype(np.float64)
    l_zero = float(np.mean(1.0 - np.abs(np.exp(-1j * r).mean(axis=1))))
    return l_net, l_zero


def image_entropy(img):
    """E = -sum p ln p, p = I^2 / sum I^2 (float64)."""
    a = np.asarray(img, np.float64).ravel() ** 2
    p = a / a.sum()
    p = p[p > 0]
    return float(-(p * np.log(p)).sum())


def evaluate_autofocus(torch, params, kind, n, tol=1e-6, cluster=16, seed0=EVAL_SEED0):
    """Per frame: the reference's autofocus (Doppler-tracking start, 120
    iterations) and the judged warm start (the learned leg until the stop
    criterion `tol`, the plain leg = the reference's autofocus, the lower
    final image entropy kept).  Returns per frame the iterations of both legs,
    their entropies of the selected bins, which leg was kept and the final
    image entropies."""
    w = workload(kind)
    M, N = w["M"], w["N"]
    s = torch.cuda.current_stream()
    x = torch.empty((M, 2 * N), dtype=torch.float32, device="cuda")
    v = torch.empty(M, dtype=torch.float64, device="cuda")
    img = torch.empty((M, 512), dtype=torch.float32, device="cuda")
    net = WSNet(M, training=False)
    net.set_params(params)
    rng = np.random.default_rng(seed0)
    rows = []
    with Context(radar(M, N), stream=s.cuda_stream) as ctx:
        cl = min(cluster, ctx.tuning().af_cluster_max)
        for i in range(n):
            synth_device(frame_params(kind, seed0 + i, rng), x, v, s.cuda_stream)
            res = {}
            for mode in ("ref120", "judged"):
                if mode == "ref120":
                    ctx.set_warmstart(None)
                    ctx.set_tuning(af_cluster=cl, af_tol=0.0, af_iters=120)
                else:
                    ctx.set_tuning(af_cluster=cl, af_tol=tol, af_iters=120)
                    ctx.set_warmstart(net)
                ctx.image_device(x, v, img, w["flags"])
                ctx.synchronize()
                tr = ctx.trace()
                res[mode] = dict(iters=tr["af_iterations"], entropy=image_entropy(img.cpu().numpy()),
                                 ws_used=tr["ws_used"], legs_entropy=tr["af_entropy_final"],
                                 legs_iters=tr["af_iterations_leg"])
            rows.append(res)
        ctx.set_warmstart(None)
    net.close()
    return rows


def summarize(rows):
    """Iterations of the learned leg (to the stop criterion) and of the plain
    leg (the reference's fixed count), how often the learned leg was kept,
    and the judged final image entropy against the reference's autofocus
    (negative: the network's gain)."""
    e120 = np.array([r["ref120"]["entropy"] for r in rows])
    ej = np.array([r["judged"]["entropy"] for r in rows])
    kept = np.array([r["judged"]["ws_used"] for r in rows], bool)
    it_p = np.array([r["judged"]["legs_iters"][0] for r in rows], float)
    it_l = np.array([r["judged"]["legs_iters"][1] for r in rows], float)
    d = ej - e120
    return dict(frames=len(rows), iters_plain_leg=float(it_p.mean()), iters_learned_leg=float(it_l.mean()),
                learned_kept_frac=float(kept.mean()),
                dE_judged_vs_ref120_max=float(d.max()), dE_judged_vs_ref120_mean=float(d.mean()),
                dE_kept_frames_mean=float(d[kept].mean()) if kept.any() else 0.0)


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--out", required=True)
    ap.add_argument("--n-poly", type=int, default=200000)
    ap.add_argument("--n-full", type=int, default=2000)
    ap.add_argument("--epochs", type=int, default=40)
    ap.add_argument("--eval", type=int, default=32)
    ap.add_argument("--report", default=None)
    a = ap.parse_args()
    import torch
    t0 = time.time()
    sets = []
    Xp, Rp, _ = make_dataset(torch, "poly", a.n_poly, TRAIN_SEED0)
    sets.append((Xp, Rp))
    if a.n_full > 0:
        Xf, Rf, _ = make_dataset(torch, "full", a.n_full, TRAIN_SEED0 + 10_000_000)
        sets.append((Xf, Rf))
    t_data = time.time() - t0
    params, hist = train(torch, sets, epochs=a.epochs)
    np.save(a.out, params)
    rep = dict(data_s=t_data, train_s=time.time() - t0 - t_data, loss_hist=hist)
    Xe, Re, _ = make_dataset(torch, "poly", 512, EVAL_SEED0 + 777)
    rep["heldout_poly"] = dict(zip(("loss_net", "loss_doppler"), eval_loss(torch, params, Xe, Re)))
    if a.n_full > 0:
        Xe, Re, _ = make_dataset(torch, "full", 64, EVAL_SEED0 + 888)
        rep["heldout_full"] = dict(zip(("loss_net", "loss_doppler"), eval_loss(torch, params, Xe, Re)))
    if a.eval > 0:
        rep["autofocus_poly"] = summarize(evaluate_autofocus(torch, params, "poly", a.eval))
        if a.n_full > 0:
            rep["autofocus_full"] = summarize(evaluate_autofocus(torch, params, "full", max(4, a.eval // 4)))
    s = json.dumps(rep, indent=1)
    print(s)
    if a.report:
        with open(a.report, "w") as f:
            f.write(s)


if __name__ == "__main__":
    main()
