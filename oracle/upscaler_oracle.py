"""Test infrastructure: CPU FP32 oracle of the learned 2x upscaler (the network of include/swlearn.h).

Used only by tests and the smoke check, as the checker of the GPU kernels; nothing in the product
calls it. The network has no counterpart in the reference (its FrameUpscaler,
src/square_wheel/frame_upscaler.rs, only has nearest and 2x-averaging upscales), so this is the
definition the GPU path is checked against:

  x = bf16((b, g, r) / 255)                      3 channels, zero padding around the image
  A_l = bf16(relu(conv3x3(A_{l-1}, bf16(W_l)) + b_l))   l = 0, 1, 2 (32 channels)
  R = conv3x3(A_2, bf16(W_3)) + b_3              12 channels, f32
  out(2x+sx, 2y+sy, c) = bilinear(x_bytes)(...) + R[c*4 + sy*2 + sx]

bf16 rounding is applied exactly where the GPU stores bf16 (activations, loss gradient, masked input
gradients, weights), so GPU and oracle differ only by FP32 summation order.
Loss: 0.5 * sum(diff^2) / n over each crop's window inset by `margin`; gradients in the canonical
layout (per layer: weights [co][ky][kx][ci], then bias [co]).
"""
import numpy as np

LAYERS = [(3, 32), (32, 32), (32, 32), (32, 12)]
NUM_PARAMS = sum(co * 9 * ci + co for ci, co in LAYERS)


def bf16(a):
    """Round float32 to the nearest bfloat16 (ties to even), returned as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32)


def split_params(p):
    out, off = [], 0
    for ci, co in LAYERS:
        nw = co * 9 * ci
        w = np.asarray(p[off:off + nw], np.float32).reshape(co, 3, 3, ci)
        b = np.asarray(p[off + nw:off + nw + co], np.float32)
        out.append((w, b))
        off += nw + co
    return out


def channels(frame):
    """Color32 (h, w) uint32 -> (h, w, 3) float32 byte values in lane order b, g, r."""
    f = frame.astype(np.uint32)
    return np.stack([(f >> s) & 255 for s in (0, 8, 16)], axis=-1).astype(np.float32)


def conv3x3(x, w):
    """x (h, w, ci), w (co, 3, 3, ci) -> (h, w, co), zero padding, float64 accumulation."""
    h, wd, ci = x.shape
    xp = np.zeros((h + 2, wd + 2, ci), np.float64)
    xp[1:-1, 1:-1] = x
    out = np.zeros((h, wd, w.shape[0]), np.float64)
    for ky in range(3):
        for kx in range(3):
            out += xp[ky:ky + h, kx:kx + wd] @ w[:, ky, kx, :].astype(np.float64).T
    return out


def conv3x3_transpose(g, w):
    """Gradient of conv3x3 w.r.t. its input: g (h, w, co), w (co, 3, 3, ci) -> (h, w, ci)."""
    h, wd, co = g.shape
    gp = np.zeros((h + 2, wd + 2, co), np.float64)
    gp[1:-1, 1:-1] = g
    out = np.zeros((h, wd, w.shape[3]), np.float64)
    for ky in range(3):
        for kx in range(3):
            # input pixel q receives g[q - (ky-1, kx-1)] * w[:, ky, kx, :]
            out += gp[2 - ky:2 - ky + h, 2 - kx:2 - kx + wd] @ w[:, ky, kx, :].astype(np.float64)
    return out


def conv3x3_wgrad(x, g):
    """dW[co, ky, kx, ci] = sum_p g[p, co] * x[p + (ky-1, kx-1), ci] (zero padding)."""
    h, wd, ci = x.shape
    xp = np.zeros((h + 2, wd + 2, ci), np.float64)
    xp[1:-1, 1:-1] = x
    gw = g.reshape(-1, g.shape[2]).astype(np.float64)
    dw = np.zeros((g.shape[2], 3, 3, ci), np.float64)
    for ky in range(3):
        for kx in range(3):
            dw[:, ky, kx, :] = gw.T @ xp[ky:ky + h, kx:kx + wd].reshape(-1, ci)
    return dw


def bilinear_base(lo_bytes, x0, y0, w, h):
    """Base image of the window (x0, y0, w, h) of the source: (h, w, 2, 2, 3) indexed [y, x, sy, sx, c],
    f32 with the GPU's operation order."""
    H, W, _ = lo_bytes.shape
    ys = np.arange(y0, y0 + h)
    xs = np.arange(x0, x0 + w)
    out = np.zeros((h, w, 2, 2, 3), np.float32)
    q = np.float32(0.75)
    r = np.float32(0.25)
    inv = np.float32(1.0 / 255.0)
    for sy in range(2):
        y1 = np.clip(ys + (1 if sy else -1), 0, H - 1)
        for sx in range(2):
            x1 = np.clip(xs + (1 if sx else -1), 0, W - 1)
            p00 = lo_bytes[ys][:, xs]
            p01 = lo_bytes[ys][:, x1]
            p10 = lo_bytes[y1][:, xs]
            p11 = lo_bytes[y1][:, x1]
            top = (q * p00).astype(np.float32) + (r * p01).astype(np.float32)
            bot = (q * p10).astype(np.float32) + (r * p11).astype(np.float32)
            v = (q * top).astype(np.float32) + (r * bot).astype(np.float32)
            out[:, :, sy, sx, :] = (v * inv).astype(np.float32)
    return out


def _ident(a):
    return np.asarray(a, np.float64)


def forward(params, lo, x0=0, y0=0, w=None, h=None, exact=False):
    """Network on the window of the Color32 frame `lo`: returns (activations, residual R (h, w, 12),
    base (h, w, 2, 2, 3)). exact=True: no bf16 rounding and float64 throughout (the differentiable
    function the finite-difference check of the backward pass uses)."""
    H, W = lo.shape
    w = W if w is None else w
    h = H if h is None else h
    q, ft = (_ident, np.float64) if exact else (bf16, np.float32)
    lb = channels(lo)
    x = q(lb[y0:y0 + h, x0:x0 + w] * ft(1.0 / 255.0))
    layers = split_params(params)
    acts = [x]
    a = x
    for l in range(3):
        wl, bl = layers[l]
        a = q(np.maximum(conv3x3(a, q(wl)).astype(ft) + bl, 0.0))
        acts.append(a)
    w3, b3 = layers[3]
    res = conv3x3(a, q(w3)).astype(ft) + b3
    return acts, res, bilinear_base(lb, x0, y0, w, h)


def predict(res, base):
    """(h, w, 12) residual + (h, w, 2, 2, 3) base -> (2h, 2w, 3) prediction in [0, 1] units."""
    h, w, _ = res.shape
    r = res.reshape(h, w, 3, 2, 2).transpose(0, 1, 3, 4, 2)  # [y, x, sy, sx, c]
    p = (base + r).astype(res.dtype)
    return p.transpose(0, 2, 1, 3, 4).reshape(2 * h, 2 * w, 3)


def infer(params, lo):
    """Full-frame inference -> Color32 (2H, 2W), alpha copied from the source pixel."""
    _, res, base = forward(params, lo)
    p = predict(res, base)
    b = np.clip(np.rint(p * np.float32(255.0)), 0, 255).astype(np.uint32)
    H, W = lo.shape
    alpha = np.repeat(np.repeat(lo.astype(np.uint32) & 0xFF000000, 2, axis=0), 2, axis=1)
    return alpha | (b[..., 2] << 16) | (b[..., 1] << 8) | b[..., 0]


def gradients(params, crops, crop_w=128, crop_h=64, margin=4, exact=False):
    """crops: list of (lo, hi, x, y) with lo/hi Color32 arrays. Returns (grads (NUM_PARAMS,), loss)."""
    q, ft = (_ident, np.float64) if exact else (bf16, np.float32)
    layers = split_params(params)
    total = [np.zeros((co, 3, 3, ci)) for ci, co in LAYERS]
    total_b = [np.zeros(co) for _, co in LAYERS]
    sq = 0.0
    n = 0
    for lo, hi, x0, y0 in crops:
        acts, res, base = forward(params, lo, x0, y0, crop_w, crop_h, exact)
        pred = predict(res, base)
        tgt = channels(hi[2 * y0:2 * (y0 + crop_h), 2 * x0:2 * (x0 + crop_w)]) * ft(1.0 / 255.0)
        diff = (pred - tgt.astype(ft)).astype(ft)
        mask = np.zeros((crop_h, crop_w), bool)
        mask[margin:crop_h - margin, margin:crop_w - margin] = True
        mask2 = np.repeat(np.repeat(mask, 2, axis=0), 2, axis=1)
        diff[~mask2] = 0.0
        sq += float(np.sum(diff.astype(np.float64) ** 2))
        n += int(mask.sum()) * 12
        # back to the 12 residual channels: channel c*4 + sy*2 + sx
        g = diff.reshape(crop_h, 2, crop_w, 2, 3).transpose(0, 2, 4, 1, 3).reshape(crop_h, crop_w, 12)
        g = q(g)
        for l in range(3, -1, -1):
            total[l] += conv3x3_wgrad(acts[l], g)
            total_b[l] += g.reshape(-1, g.shape[2]).sum(axis=0)
            if l == 0:
                break
            gin = conv3x3_transpose(g, q(layers[l][0]))
            g = q((gin * (acts[l] > 0)).astype(ft))
    out = []
    for l in range(4):
        out.append((total[l] / n).astype(ft).ravel())
        out.append((total_b[l] / n).astype(ft))
    return np.concatenate(out), 0.5 * sq / n


def loss(params, crops, crop_w=128, crop_h=64, margin=4, exact=True):
    """The loss alone (for finite differences)."""
    sq, n = 0.0, 0
    ft = np.float64 if exact else np.float32
    for lo, hi, x0, y0 in crops:
        _, res, base = forward(params, lo, x0, y0, crop_w, crop_h, exact)
        pred = predict(res, base)
        tgt = channels(hi[2 * y0:2 * (y0 + crop_h), 2 * x0:2 * (x0 + crop_w)]) * ft(1.0 / 255.0)
        diff = pred - tgt
        d = diff[2 * margin:2 * (crop_h - margin), 2 * margin:2 * (crop_w - margin)]
        sq += float(np.sum(d.astype(np.float64) ** 2))
        n += (crop_h - 2 * margin) * (crop_w - 2 * margin) * 12
    return 0.5 * sq / n
