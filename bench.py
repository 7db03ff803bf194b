"""Benchmark: frames/s of the ISAR imaging chain at 1024 pulses x 8192 range
cells complex64, the full five-stage workload (high-speed compensation, range
alignment, centring + cut, fast minimum-entropy autofocus, CZT MTRC).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Headline (`value`): the batched pipeline.  A step is one batch of B = 128
distinct frames imaged by one CUDA graph (isar_batch_run: per-shape lanes,
cluster-resident autofocus), inputs resident in HBM (8 GiB > L2).  Three
autofocus arms are tried in order and the first whose images pass the
equal-entropy check is timed: (1) the learned warm start judged by the plain
autofocus (the autofocus runs from the network's start until the entropy stop
criterion and, as the reference does, from the Doppler-tracking start for 120
iterations; both are imaged and the lower final image entropy is kept), (2)
the stop criterion alone (Doppler-tracking start), (3) the reference
algorithm (120 iterations).  The check, per frame: no
frame's final image entropy may exceed the plain pipeline's on the same frame
by more than 1e-4.  Every arm's check is reported.
`plain` is the single-frame pipeline (isar_image_device, the reference's
algorithm: 120 autofocus iterations on the context's default engine), timed
the same way.
`e2e` goes through the public C ABI with pinned host buffers: every step
copies its 128 echoes host->device as int16 I/Q samples (the sensor format, 4
bytes per sample; range alignment reads them directly) and reads the 128
images back, eight buffer sets in rotation so that the copies of the next
steps overlap the current step's compute (beside the running batch about one
host->device copy in seven takes ~0.2 s instead of 20 ms; eight sets give the
copies ~0.45 s of slack), over at least E2E_MIN_STEPS steps so that the
first step's copy, which starts from idle streams, does not dominate the
streaming rate.  Under torchrun every rank images its own frames (replicas,
weak scaling).

--impl reference times the CPU restatement of the reference's chain (the
oracle) on all host cores, one frame per worker process per step.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

M, N = 1024, 8192
C = 512
B = 128                     # frames per batch step
TOL = 3e-7                  # autofocus entropy stop criterion (relative change per iteration)
TOL_LEARNED = 1e-5          # the learned leg's stop criterion (on 256 frames its judged gain is the same as at 3e-6
                            # and 3e-7; 59 iterations against 71 and 98)
E2E_SETS = 8                # end-to-end buffer sets in rotation (copies of later steps run ahead)
E2E_CHUNKS = 16             # host->device copy of a step in this many pieces
E2E_MIN_STEPS = 120         # end-to-end steps at least: the streaming rate, not the pipeline's fill
METRIC = "frames/s @1024×8192 c64: learned+batched vs plain on 1 GB300, equal entropy"
ARMS = [("learned warm start (to the entropy stop criterion) judged against the plain autofocus (120 iterations) "
         "on final image entropy", True, TOL_LEARNED),
        ("entropy stop criterion, Doppler-tracking start", False, TOL),
        ("reference algorithm (120 iterations)", False, 0.0)]
WORKLOAD = ("full five-stage pipeline, 1024 pulses x 8192 range cells complex64, HPC + MTRC on, "
            "batches of 128 frames")
# DRAM bytes (read + write) of one range-alignment stage at 1024 x 8192, all
# its kernels, per frame (spectral envelope merge): dram__bytes_read.sum +
# dram__bytes_write.sum from an ncu capture of `bench.py --profile plain`
# (two frames, halved); writes still in L2 at a kernel's end are not counted
RA_STAGE_TRAFFIC = 251913088


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("BENCH_BACKEND", "nccl") == "nccl" else "gloo")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(ws, v, device):
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi during a region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.p = None
        self.rows = []

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "100"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.p = None

    def _read(self):
        for line in self.p.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.t.join(timeout=2)
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows if len(r) >= 9 for i in range(4)
                          if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(sm)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ra_algorithmic_bytes(M, N):
    """Compulsory HBM bytes of range alignment as this project formulates it
    (spectral envelope merge): level 0 reads all M rows (8MN) and stores the
    M/2 merged group spectra (N complex each, 4MN); level l >= 1 reads its
    M/2^l group spectra and, below the last level, stores M/2^(l+1) merged
    ones; the final transform reads and writes every row (16MN)."""
    L = M.bit_length() - 1
    b = 8 * M * N + (4 * M * N if L > 1 else 0) + 16 * M * N
    for lv in range(1, L):
        b += (M >> lv) * N * 8
        if lv < L - 1:
            b += (M >> (lv + 1)) * N * 8
    return b


def image_entropy(img):
    import numpy as np
    a = np.asarray(img, np.float64).ravel() ** 2
    p = a / a.sum()
    p = p[p > 0]
    return float(-(p * np.log(p)).sum())


def run_gb300(args):
    import numpy as np
    import torch

    import isar_imaging_cuda_gb300 as g

    ws, rank, local = dist_init()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    s = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(s)
    stream = s.cuda_stream
    rp = g.radar(M, N)
    flags = g.FLAG_HPC | g.FLAG_MTRC
    X = torch.empty((B, M, 2 * N), dtype=torch.float32, device=dev)
    V = torch.empty((B, M), dtype=torch.float64, device=dev)
    for i in range(B):
        g.synth_device(g.synth_params(M, N, seed=1000 * rank + i, full=True), X[i], V[i], stream)

    def ev():
        return torch.cuda.Event(enable_timing=True)

    # ---- plain single-frame pipeline (the reference's algorithm) ----
    ctx = g.Context(rp, device=local, stream=stream)
    img = torch.empty((M, C), dtype=torch.float32, device=dev)
    e_plain = []
    for i in range(B):
        ctx.image_device(X[i], V[i], img, flags)
        ctx.synchronize()
        e_plain.append(image_entropy(img.cpu().numpy()))
    for i in range(args.warmup):
        ctx.image_device(X[i % B], V[i % B], img, flags)
    s.synchronize()
    barrier(ws)
    e0, e1 = ev(), ev()
    e0.record(s)
    for i in range(args.steps):
        ctx.image_device(X[i % B], V[i % B], img, flags)
    e1.record(s)
    s.synchronize()
    ctx.synchronize()
    plain_ms = max_over_ranks(ws, e0.elapsed_time(e1) / args.steps, dev)

    # per-stage times of the plain pipeline (stage entry points on a copy)
    scratch = torch.empty_like(X[0])
    cut = torch.empty((M, 2 * C), dtype=torch.float32, device=dev)
    img2 = torch.empty((M, C), dtype=torch.float32, device=dev)
    stage = {"range_align": [], "center_cut": [], "fast_entropy": [], "mtrc_post": []}
    for i in range(args.warmup + min(args.steps, 10)):
        scratch.copy_(X[i % B])
        ev_ = [ev() for _ in range(5)]
        ev_[0].record(s)
        ctx.stage_range_align(scratch, V[i % B], g.FLAG_HPC)
        ev_[1].record(s)
        ctx.stage_center_cut(scratch, cut)
        ev_[2].record(s)
        ctx.stage_fast_entropy(cut, 120)
        ev_[3].record(s)
        ctx.stage_post(cut, img2, g.FLAG_MTRC)
        ev_[4].record(s)
        s.synchronize()
        if i >= args.warmup:
            for k, name in enumerate(stage):
                stage[name].append(ev_[k].elapsed_time(ev_[k + 1]))
    stage_ms = {k: statistics.median(v) for k, v in stage.items()}
    U = int(ctx.trace()["unit2_num"])
    cl0 = ctx.tuning().af_cluster
    plain_engine = "cooperative grid" if cl0 == 0 else "cluster of %d CTAs" % cl0
    ctx.close()

    # ---- headline: batched + learned warm start + stop criterion ----
    net = g.WSNet(M, training=False, device=local, stream=stream)
    net.load_params(g.WARMSTART_WEIGHTS)
    imgs = torch.empty((B, M, C), dtype=torch.float32, device=dev)
    lst = g.Batch.frames((rp, X[i], V[i], flags, imgs[i]) for i in range(B))
    batch = g.Batch(device=local, stream=stream)
    cl = 16
    probe = g.Context(rp, device=local, stream=stream)
    cl = min(cl, probe.tuning().af_cluster_max)
    probe.close()

    def configure(learned, tol):
        t = g.Tuning(ra_pair_min=128, ra_rows_per_cta=4, ra_rows_final=4, af_cluster=cl,
                     af_tol=tol, af_iters=120, af_cluster_max=0)
        batch.set_warmstart(net if learned else None)
        batch.set_tuning(rp, t)
        tune_ms = batch.autotune(lst)
        batch.run(lst)
        batch.synchronize()
        ent = [image_entropy(imgs[i].cpu().numpy()) for i in range(B)]
        return tune_ms, ent

    # first arm whose images pass the equal-entropy check (the last one is
    # the reference algorithm itself)
    check = {"criterion": "every frame: final image entropy <= the plain pipeline's + 1e-4", "frames": B,
             "arms": []}
    for name, learned, tol in ARMS:
        tune_ms, e_batch = configure(learned, tol)
        dE = np.array(e_batch) - np.array(e_plain)
        ok = bool(dE.max() <= 1e-4)
        check["arms"].append({"arm": name, "tol": tol, "mean_dE": float(dE.mean()), "max_dE": float(dE.max()),
                              "min_dE": float(dE.min()), "frames_worse_1e-4": int((dE > 1e-4).sum()),
                              "passed": ok})
        if ok or tol == 0.0:
            break
    mode = "batched, " + name
    learned_timed = learned
    lanes = batch.lanes()
    tuning = batch.tuning(rp).as_dict()

    for _ in range(args.warmup):
        batch.run(lst)
    s.synchronize()
    barrier(ws)
    clocks = Clocks(local)
    clocks.start()
    n0 = g.launch_count()
    e0, e1 = ev(), ev()
    e0.record(s)
    for _ in range(args.steps):
        batch.run(lst)
    e1.record(s)
    s.synchronize()
    batch.synchronize()
    launches = (g.launch_count() - n0) // max(args.steps, 1)
    ms = e0.elapsed_time(e1) / args.steps
    clk = clocks.stop()
    ms = max_over_ranks(ws, ms, dev)
    barrier(ws)

    # ---- end to end: pinned host echoes in, images out, E2E_SETS buffer sets ----
    # The echoes travel as the sensor's int16 I/Q samples (the frames are
    # int16-quantised: the same samples) and range alignment reads them
    # directly (ISAR_FLAG_IQ16).
    HQ = torch.empty((B, M, 2 * N), dtype=torch.int16, pin_memory=True)
    HQ.copy_(X.to(torch.int16).cpu())
    HV = V.cpu().pin_memory()
    Q = [torch.empty((B, M, 2 * N), dtype=torch.int16, device=dev) for _ in range(E2E_SETS)]
    fq = flags | g.FLAG_IQ16
    HI = [torch.empty((B, M, C), dtype=torch.float32, pin_memory=True) for _ in range(E2E_SETS)]
    Vs = [V] + [torch.empty_like(V) for _ in range(E2E_SETS - 1)]
    Is = [imgs] + [torch.empty_like(imgs) for _ in range(E2E_SETS - 1)]
    sets = [(Q[k], Vs[k], Is[k], g.Batch.frames((rp, Q[k][i], Vs[k][i], fq, Is[k][i]) for i in range(B)))
            for k in range(E2E_SETS)]
    # three streams: host->device copies (cs), the batch (s), device->host
    # copies (ds); buffer set i % E2E_SETS is reused E2E_SETS steps later
    cs = torch.cuda.Stream(device=dev)
    ds = torch.cuda.Stream(device=dev)
    h2d_done = [torch.cuda.Event() for _ in range(E2E_SETS)]
    run_done = [torch.cuda.Event() for _ in range(E2E_SETS)]
    d2h_done = [torch.cuda.Event() for _ in range(E2E_SETS)]
    for e in run_done + d2h_done:
        e.record(s)

    def e2e_step(i):
        k = i % E2E_SETS
        Qd, Vd, Id, L = sets[k]
        cs.wait_event(run_done[k])           # the set's previous batch has consumed Qd, Vd
        with torch.cuda.stream(cs):
            for q in range(E2E_CHUNKS):
                sl = slice(q * B // E2E_CHUNKS, (q + 1) * B // E2E_CHUNKS)
                Qd[sl].copy_(HQ[sl], non_blocking=True)
            Vd.copy_(HV, non_blocking=True)
            h2d_done[k].record(cs)
        s.wait_event(h2d_done[k])
        s.wait_event(d2h_done[k])            # the set's previous images are read back
        batch.run(L)
        run_done[k].record(s)
        ds.wait_event(run_done[k])
        with torch.cuda.stream(ds):
            HI[k].copy_(Id, non_blocking=True)
            d2h_done[k].record(ds)

    # the host->device bandwidth of this machine now (one step's int16 echoes
    # alone): the end-to-end rate is bounded by it when it falls below the
    # batch's consumption rate
    torch.cuda.synchronize()
    h2d_t = []
    for _ in range(3):   # the first copy also pays one-time mapping costs
        h0, h1 = ev(), ev()
        h0.record(cs)
        with torch.cuda.stream(cs):
            Q[0].copy_(HQ, non_blocking=True)
        h1.record(cs)
        cs.synchronize()
        h2d_t.append(h0.elapsed_time(h1))
    h2d_alone_ms = statistics.median(h2d_t)
    for i in range(max(args.warmup, E2E_SETS)):   # every set's graph is captured before timing
        e2e_step(i)
    torch.cuda.synchronize()
    barrier(ws)
    # The timed loop starts with every stream idle, so its first step waits
    # for a whole host->device copy, which next to the running batch graph
    # can take ~0.2 s instead of 20 ms (measured: copies alone never do;
    # beside the batch about one in seven does, and once the copies run
    # ahead the buffer sets absorb it).  Enough steps keep that one-time
    # fill from dominating the streaming rate.
    e2e_steps = max(args.steps, E2E_MIN_STEPS)
    clocks_e2e = Clocks(local)
    clocks_e2e.start()
    t0 = time.perf_counter()
    for i in range(e2e_steps):
        e2e_step(i)
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(ws, (time.perf_counter() - t0) / e2e_steps, dev)
    clk_e2e = clocks_e2e.stop()
    batch.synchronize()

    peak, peak_kind = peaks()
    ra_bytes = ra_algorithmic_bytes(M, N)
    roof = {"kernel": "range alignment, 1024 x 8192 (k_ra_spec0 + k_ra_spec levels + k_ra_final, spectral "
                      "envelope merge, HPC fused), single frame", "bound": "hbm",
            "achieved": ra_bytes / (stage_ms["range_align"] * 1e-3) / 1e9, "algorithmic_bytes": ra_bytes,
            "ms": stage_ms["range_align"], "peak": peak, "unit": "GB/s", "peak_kind": peak_kind,
            "traffic": RA_STAGE_TRAFFIC}
    roof["frac"] = roof["achieved"] / peak

    out = {
        "metric": METRIC,
        "value": ws * B * 1e3 / ms,
        "unit": "frames/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "c64 (fp32 complex); warm-start network bf16 with fp32 accumulate",
        "data": "synthetic: seeded dechirped LFM echoes generated on the GPU (200 scatterers, 40 m x 40 m, "
                "4 deg rotation, 3000 m/s + 50 m/s^2, drift 0.5 cell, quadratic+random phase error, SNR 5 dB)",
        "config": {"workload": WORKLOAD, "pipeline": mode, "M": M, "N": N, "flags": "hpc+mtrc",
                   "batch_frames": B, "lanes": lanes, "tuning": tuning, "autotune_best_ms": tune_ms,
                   "l2": "inputs larger than L2: 128 distinct frames x 64 MiB per step", "parallelism": "replicas"},
        "plain": {"frames_per_s": ws * 1e3 / plain_ms, "ms_per_frame": plain_ms, "stage_ms": stage_ms, "U": U,
                  "pipeline": "single frame per call, the reference's algorithm (120 autofocus iterations), "
                              "default autofocus engine: " + plain_engine},
        "speedup_vs_plain": plain_ms * B / ms,
        "entropy_check": check,
        "e2e": {"value": ws * B / e2e_s, "unit": "frames/s", "h2d_bytes_per_step": B * (M * N * 4 + M * 8),
                "d2h_bytes_per_step": B * M * C * 4,
                "input": "int16 I/Q echoes (the sensor format), read directly by range alignment (ISAR_FLAG_IQ16)",
                "ms_per_step": e2e_s * 1e3, "steps": e2e_steps, "h2d_alone_ms": h2d_alone_ms, "clocks": clk_e2e,
                "h2d_gbs": B * M * N * 4 / (h2d_alone_ms * 1e-3) / 1e9},
        "roofline": roof,
        "gpu_launches": int(launches),
        "clocks": clk,
    }
    # context: the same batch and lanes with the reference's autofocus alone
    # (no network, 120 iterations), i.e. what the judged warm start costs
    ref_batch = None
    if learned_timed:
        t_ref = batch.tuning(rp)
        t_ref.af_tol = 0.0
        batch.set_warmstart(None)
        batch.set_tuning(rp, t_ref)
        for _ in range(2):
            batch.run(lst)
        s.synchronize()
        r0, r1 = ev(), ev()
        r0.record(s)
        for _ in range(max(args.steps // 2, 3)):
            batch.run(lst)
        r1.record(s)
        s.synchronize()
        ref_ms = r0.elapsed_time(r1) / max(args.steps // 2, 3)
        ref_batch = {"frames_per_s": B * 1e3 / ref_ms, "ms_per_step": ref_ms,
                     "pipeline": "batched, reference autofocus alone (Doppler-tracking start, 120 iterations), "
                                 "same lanes and tuning"}
    batch.close()
    net.close()
    if rank == 0 and not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(X[0], V[0])
    if rank == 0:
        del X, Vs, Is, imgs, HQ, Q, sets
        torch.cuda.empty_cache()
        out["other_workloads"] = other_workloads(g, torch, s, args.steps)
        if ref_batch is not None:
            out["other_workloads"]["batch128_reference_autofocus"] = ref_batch
    if rank == 0:
        print(json.dumps(out))


def other_workloads(g, torch, s, steps):
    """The other configurations: the plain 256 x 4096 workload (single frame
    per call, and batches of 32 frames), 64 frames of uneven size (pulses
    uniform over {128, 256, 512, 1024}, range cells over {2048, 4096, 8192},
    plain-workload scenes) in one batch graph, and the IFDS ingest's pulse
    compression (1024 pulses of 5000 samples in one launch)."""
    import numpy as np

    def timed(fn, reps):
        for _ in range(2):
            fn()
        s.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(reps):
            fn()
        e1.record(s)
        s.synchronize()
        return e0.elapsed_time(e1) / reps

    out = {}
    # plain workload, 256 pulses x 4096 range cells, no HPC / MTRC
    m1, n1, b1 = 256, 4096, 32
    rp1 = g.radar(m1, n1)
    X = torch.empty((b1, m1, 2 * n1), dtype=torch.float32, device="cuda")
    img = torch.empty((b1, m1, C), dtype=torch.float32, device="cuda")
    for i in range(b1):
        g.synth_device(g.synth_params(m1, n1, seed=5000 + i), X[i], None, s.cuda_stream)
    with g.Context(rp1, stream=s.cuda_stream) as ctx:
        k = [0]

        def one():
            ctx.image_device(X[k[0] % b1], None, img[k[0] % b1], 0)
            k[0] += 1
        ms1 = timed(one, max(steps, 10))
    with g.Batch(stream=s.cuda_stream) as b:
        lst = g.Batch.frames((rp1, X[i], None, 0, img[i]) for i in range(b1))
        b.autotune(lst)
        msb = timed(lambda: b.run(lst), max(steps // 2, 3))
        lanes = b.lanes()
    out["plain_256x4096"] = {"single_frame_frames_per_s": 1e3 / ms1, "batch32_frames_per_s": b1 * 1e3 / msb,
                             "batch_lanes": lanes}
    del X, img
    # 64 frames of uneven size in one batch graph
    rng = np.random.default_rng(2024)
    Ms = rng.choice([128, 256, 512, 1024], 64)
    Ns = rng.choice([2048, 4096, 8192], 64)
    frames, keep = [], []
    for i, (m, n) in enumerate(zip(Ms, Ns)):
        m, n = int(m), int(min(max(n, m), 8192))
        x = torch.empty((m, 2 * n), dtype=torch.float32, device="cuda")
        im = torch.empty((m, C), dtype=torch.float32, device="cuda")
        g.synth_device(g.synth_params(m, n, seed=7000 + i), x, None, s.cuda_stream)
        keep += [x, im]
        frames.append((g.radar(m, n), x, None, 0, im))
    with g.Batch(stream=s.cuda_stream) as b:
        lst = g.Batch.frames(frames)
        b.autotune(lst)
        msu = timed(lambda: b.run(lst), max(steps // 2, 3))
        lanes = b.lanes()
    out["uneven_batch64"] = {"frames_per_s": 64 * 1e3 / msu, "ms_per_batch": msu, "lanes_per_shape": lanes,
                             "shapes": len({(int(a), int(c)) for a, c in zip(Ms, Ns)}),
                             "pulse_cells": int(sum(int(a) * int(c) for a, c in zip(Ms, Ns)))}
    del keep, frames
    # IFDS ingest: pulse compression of 1024 pulses of 5000 samples (NFFT
    # 8192: three 8192-point transforms per pulse) in one launch; random
    # int16 samples (the cost does not depend on the data)
    P, L, NF = 1024, 5000, 8192
    rpi = g.radar(1024, 4096, B=100e6, fc=10e9, Fs=200e6, Tp=10e-6, data_type=g.IFDS)
    gen = torch.Generator(device="cuda")
    gen.manual_seed(11)
    ad = torch.randint(-2000, 2000, (P, 2 * L), dtype=torch.int16, device="cuda", generator=gen)
    vel = torch.linspace(-300.0, 300.0, P, dtype=torch.float64, device="cuda")
    pc_out = torch.empty((P, 4096, 2), dtype=torch.float32, device="cuda")
    with g.Context(rpi, stream=s.cuda_stream) as ctx:
        msp = timed(lambda: ctx.pulse_compress(ad, L, vel, pc_out), max(steps, 10))
    out["ifds_pulse_compression"] = {"pulses_per_s": P * 1e3 / msp, "ms_per_launch": msp, "pulses": P,
                                     "iq_len": L, "nfft": NF,
                                     "fft_gflop_per_s": P * 3 * 5 * NF * 13 / (msp * 1e-3) / 1e9}
    return out


def cpu_model():
    """The host CPU's model name (x86 /proc/cpuinfo, else lscpu, as on Arm)."""
    try:
        with open("/proc/cpuinfo") as fh:
            for line in fh:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    try:
        import subprocess
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    import platform
    return platform.machine()


def cpu_baseline(frame, vel):
    """FP64 oracle on one frame of the same workload (bounded sample)."""
    import numpy as np

    import oracle
    e = frame.cpu().numpy().view(np.complex64)
    v = vel.cpu().numpy()
    t0 = time.perf_counter()
    oracle.image(e, v, oracle.radar(M, N), hpc=True, mtrc=True)
    dt = time.perf_counter() - t0
    return {"value": 1.0 / dt, "unit": "frames/s", "cores": 1, "cpu_model": cpu_model(), "kind": "port",
            "sample": "1 frame of the 1024x8192 five-stage workload, FP64 oracle, 1 thread (%.1f s)" % dt}


_REF = {}


def _ref_init(e, vel):
    _REF["e"], _REF["v"] = e, vel


def _ref_frame(_):
    import oracle
    t0 = time.perf_counter()
    oracle.image(_REF["e"], _REF["v"], oracle.radar(M, N), hpc=True, mtrc=True)
    return time.perf_counter() - t0


def run_reference(args):
    ws, rank, _ = dist_init()
    if rank != 0:
        return
    import multiprocessing as mp

    import numpy as np

    import oracle
    # the timed workload's scene (200 scatterers): the autofocus cost follows
    # the number of selected range bins, which the scene sets; the synthesis
    # (about a minute on one core) runs once, before the timed steps
    iq, vel = oracle.synth(dict(M=M, N=N, n_scat=200, seed=7, patch_x=40.0, patch_y=40.0, drift_sigma=0.5,
                                phase_uniform=0.5, phase_quad=6.0, v0=3000.0, accel=50.0, snr_db=5.0,
                                omega=np.deg2rad(4.0) / (M / 1000.0)))
    e = oracle.iq_to_c64(iq)
    cores = os.cpu_count() or 1
    steps = max(1, min(args.steps, 4))
    warm = 1
    with mp.get_context("spawn").Pool(cores, initializer=_ref_init, initargs=(e, vel)) as pool:
        walls = []
        for i in range(warm + steps):
            t0 = time.perf_counter()
            pool.map(_ref_frame, range(cores))
            if i >= warm:
                walls.append(time.perf_counter() - t0)
    v = cores / statistics.median(walls)
    sample = ("%d steps x %d frames of 1024x8192, 200 scatterers (one per worker process, FP64 oracle, "
              "1 thread each); steps capped at 4 to bound the run" % (steps, cores))
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": "frames/s", "n_gpus": ws,
           "steps": steps, "warmup": warm, "higher_is_better": True,
           "config": {"workload": "full five-stage pipeline, 1024 pulses x 8192 range cells complex64, HPC + MTRC on"},
           "cpu_baseline": {"value": v, "unit": "frames/s", "cores": cores, "cpu_model": cpu_model(), "kind": "port",
                            "sample": sample},
           "e2e": {"value": v, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def run_profile(args):
    """Profiling workloads (no timing, no JSON): `plain` images one
    1024 x 8192 frame warmup + steps times; `batch` runs a batch of 8 frames
    through isar_batch_run with the reference algorithm (4-CTA cluster
    autofocus, 120 iterations); `learned` the same batch with the learned
    warm start and the entropy stop criterion; `ifds` the IFDS pulse
    compression of 1024 pulses of 5000 samples and the HRRP of one
    1024 x 8192 frame."""
    import torch

    import isar_imaging_cuda_gb300 as g
    s = torch.cuda.Stream()
    torch.cuda.set_stream(s)
    rp = g.radar(M, N)
    flags = g.FLAG_HPC | g.FLAG_MTRC
    nb = 8 if args.profile in ("batch", "learned") else 1
    X = torch.empty((nb, M, 2 * N), dtype=torch.float32, device="cuda")
    V = torch.empty((nb, M), dtype=torch.float64, device="cuda")
    imgs = torch.empty((nb, M, C), dtype=torch.float32, device="cuda")
    for i in range(nb):
        g.synth_device(g.synth_params(M, N, seed=i, full=True), X[i], V[i], s.cuda_stream)
    if args.profile == "plain":
        with g.Context(rp, stream=s.cuda_stream) as ctx:
            for _ in range(args.warmup + args.steps):
                ctx.image_device(X[0], V[0], imgs[0], flags)
            ctx.synchronize()
    elif args.profile == "ifds":
        P, L = 1024, 5000
        rpi = g.radar(1024, 4096, B=100e6, fc=10e9, Fs=200e6, Tp=10e-6, data_type=g.IFDS)
        gen = torch.Generator(device="cuda")
        gen.manual_seed(11)
        ad = torch.randint(-2000, 2000, (P, 2 * L), dtype=torch.int16, device="cuda", generator=gen)
        vel = torch.linspace(-300.0, 300.0, P, dtype=torch.float64, device="cuda")
        pc_out = torch.empty((P, 4096, 2), dtype=torch.float32, device="cuda")
        hr = torch.empty_like(X[0])
        with g.Context(rpi, stream=s.cuda_stream) as ci, g.Context(rp, stream=s.cuda_stream) as cs:
            for _ in range(args.warmup + args.steps):
                ci.pulse_compress(ad, L, vel, pc_out)
                cs.stage_hrrp(X[0], hr)
            ci.synchronize()
    else:
        learned = args.profile == "learned"
        net = None
        if learned:
            net = g.WSNet(M, stream=s.cuda_stream)
            net.load_params(g.WARMSTART_WEIGHTS)
        with g.Batch(stream=s.cuda_stream, lanes=8) as b:
            if learned:
                b.set_warmstart(net)
            # the batch's autotuned configuration at 128 frames (one frame per
            # lane, 4-CTA autofocus clusters, 4 rows per CTA in the final transform)
            b.set_tuning(rp, g.Tuning(ra_pair_min=128, ra_rows_per_cta=16, ra_rows_final=4, af_cluster=4,
                                      af_tol=TOL_LEARNED if learned else 0.0, af_iters=120, af_cluster_max=0))
            lst = g.Batch.frames((rp, X[i], V[i], flags, imgs[i]) for i in range(nb))
            for _ in range(args.warmup + args.steps):
                b.run(lst)
            b.synchronize()
        if net is not None:
            net.close()
    torch.cuda.synchronize()
    print("profile workload %s done" % args.profile)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--profile", choices=["plain", "batch", "learned", "ifds"], default=None,
                    help="run a profiling workload only (for ncu), no measurement")
    args = ap.parse_args()
    if args.profile:
        run_profile(args)
        return
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
