"""FP64 CPU restatement of the learned autofocus warm-start network (test
infrastructure only: it checks the CUDA forward and backward kernels).

The reference has no learned component, so there is nothing to follow there;
this file restates the network the CUDA library implements:
  X0 [M][64] -> 6 x (1-D conv k=5 'same', 64 -> 64, bias, ReLU)
  -> 1x1 64 -> 64 + ReLU -> 1x1 64 -> 2 = (c, s),   r_hat = atan2(s, c),
  loss per frame = 1 - |mean_{m < M-1} exp(j (r_hat_m - r_m))|.
With emulate=True the values the GPU stores in bf16 (GEMM operands:
activations, weights, output gradients) are rounded to bf16 at the same
points; all sums run in float64.  The backward pass of this file is itself
pinned against central finite differences with emulate=False
(tests/test_wsnet_oracle.py).
"""
import numpy as np

CH, TAPS, NCONV = 64, 5, 6
COLK = CH * TAPS


def layer_shapes():
    """(rows, cols) of each weight matrix in canonical order."""
    return [(CH, COLK)] * NCONV + [(CH, CH), (2, CH)]


def n_params():
    return sum(r * c + r for r, c in layer_shapes())


def unpack(p):
    """Canonical flat vector -> list of (W, b) (views)."""
    out, o = [], 0
    for r, c in layer_shapes():
        W = p[o:o + r * c].reshape(r, c)
        o += r * c
        b = p[o:o + r]
        o += r
        out.append((W, b))
    assert o == p.size
    return out


def init_params(seed=0, out_scale=0.01):
    """He-normal hidden weights, zero hidden biases; a small last layer with
    bias (1, 0), so that an untrained network predicts r_hat ~ 0 (the
    Doppler-tracking start)."""
    rng = np.random.default_rng(seed)
    shapes = layer_shapes()
    parts = []
    for li, (r, c) in enumerate(shapes):
        last = li == len(shapes) - 1
        W = rng.standard_normal((r, c)) * (out_scale if last else np.sqrt(2.0 / c))
        b = np.array([1.0, 0.0]) if last else np.zeros(r)
        parts += [W.ravel(), b]
    return np.concatenate(parts).astype(np.float32)


def bf16(x):
    """Round float32 values to the nearest bfloat16 (ties to even)."""
    f = np.ascontiguousarray(x, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).reshape(f.shape)


def _r(x, emulate):
    return bf16(x).astype(np.float64) if emulate else np.asarray(x, np.float64)


def _f32(x, emulate):
    return np.asarray(x, np.float32).astype(np.float64) if emulate else x


def im2col(a):
    """a [F][M][64] -> [F][M][320], column k*64 + c = a[m + k - 2][c] (0 outside)."""
    F, M, C = a.shape
    pad = np.zeros((F, M + TAPS - 1, C), a.dtype)
    pad[:, TAPS // 2:TAPS // 2 + M] = a
    return np.concatenate([pad[:, k:k + M] for k in range(TAPS)], axis=2)


def col2im(d):
    """Adjoint of im2col: d [F][M][320] -> [F][M][64]."""
    F, M, _ = d.shape
    out = np.zeros((F, M + TAPS - 1, CH))
    for k in range(TAPS):
        out[:, k:k + M] += d[:, :, k * CH:(k + 1) * CH]
    return out[:, TAPS // 2:TAPS // 2 + M]


def forward(p, x0, emulate=True):
    """x0 [F][M][64] (bf16 values) -> out [F][M][2] and the cache."""
    L = unpack(np.asarray(p, np.float32).astype(np.float64) if emulate else np.asarray(p, np.float64))
    Wq = [(_r(W, emulate), b) for W, b in L]
    acts = [np.asarray(x0, np.float64)]
    cols = []
    a = acts[0]
    for li in range(NCONV):
        col = im2col(a)
        cols.append(col)
        z = _f32(col @ Wq[li][0].T, emulate) + Wq[li][1]
        a = _r(np.maximum(z, 0.0), emulate)
        acts.append(a)
    z = _f32(a @ Wq[NCONV][0].T, emulate) + Wq[NCONV][1]
    a = _r(np.maximum(z, 0.0), emulate)
    acts.append(a)
    out = _f32(a @ Wq[NCONV + 1][0].T, emulate) + Wq[NCONV + 1][1]
    return out, dict(acts=acts, cols=cols, Wq=Wq)


def loss_grad(p, x0, target, emulate=True):
    """Mean loss over frames and its gradient (canonical order, float64)."""
    out, cache = forward(p, x0, emulate)
    F, M, _ = out.shape
    c, s = out[..., 0], out[..., 1]
    d = np.arctan2(s, c) - target
    v = np.arange(M) < M - 1
    e = np.exp(1j * d) * v
    z = e.sum(axis=1) / (M - 1)
    az = np.abs(z)
    loss = float(np.mean(1.0 - az))
    g = (np.imag(np.conj(z)[:, None] * np.exp(1j * d)) / ((M - 1) * az[:, None] * F)) * v
    r2 = c * c + s * s
    dout = np.zeros_like(out)
    dout[..., 0] = -g * s / r2
    dout[..., 1] = g * c / r2
    acts, cols, Wq = cache["acts"], cache["cols"], cache["Wq"]
    grads = [None] * (NCONV + 2)
    dz = _r(dout, emulate)
    grads[NCONV + 1] = (np.einsum("fmo,fmk->ok", dz, acts[NCONV + 1]), dz.sum(axis=(0, 1)))
    dact = _f32(dz @ Wq[NCONV + 1][0], emulate)
    dz = _r(dact * (acts[NCONV + 1] > 0), emulate)
    grads[NCONV] = (np.einsum("fmo,fmk->ok", dz, acts[NCONV]), dz.sum(axis=(0, 1)))
    dact = _f32(dz @ Wq[NCONV][0], emulate)
    for li in range(NCONV - 1, -1, -1):
        dz = _r(dact * (acts[li + 1] > 0), emulate)
        grads[li] = (np.einsum("fmo,fmk->ok", dz, cols[li]), dz.sum(axis=(0, 1)))
        if li > 0:
            dact = col2im(_f32(dz @ Wq[li][0], emulate))
    flat = np.concatenate([np.concatenate([gw.ravel(), gb.ravel()]) for gw, gb in grads])
    return loss, flat
