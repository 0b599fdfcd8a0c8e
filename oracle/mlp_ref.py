"""FP64 CPU restatement of the learned-proposal network (TEST INFRASTRUCTURE).

Same parameter layout and maths as messi_gb300/csrc/mlp.cu: three linear
layers in -> H -> H -> out, SiLU after the first two, a K-component diagonal
Gaussian-mixture head [K logits | K*D means | K*D log-sd (clamped to
[-7, 5])] and the mean negative log-likelihood of targets.  With
``bf16=True`` weights, activations and the gradient operands of the
backward products are rounded to bfloat16 the way the GPU kernels stage them
for the tensor cores (the bias gradients are column sums of the unrounded
FP32 gradients, as on the GPU), so the comparison isolates accumulation
order.
"""
import numpy as np

LOG2PI_HALF = 0.91893853320467274


def offsets(nin, H, nout):
    o = [0]
    o.append(o[-1] + H * nin)     # b1
    o.append(o[-1] + H)           # W2
    o.append(o[-1] + H * H)       # b2
    o.append(o[-1] + H)           # W3
    o.append(o[-1] + nout * H)    # b3
    return o, o[-1] + nout


def to_bf16(a):
    """Round float32 values to bfloat16 (nearest even), returned as float64."""
    a = np.asarray(a, dtype=np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p, nin, H, nout):
    o, n = offsets(nin, H, nout)
    p = np.asarray(p, np.float64)
    return (p[o[0]:o[1]].reshape(H, nin), p[o[1]:o[2]], p[o[2]:o[3]].reshape(H, H), p[o[3]:o[4]],
            p[o[4]:o[5]].reshape(nout, H), p[o[5]:n])


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(p, x, nin, H, nout, bf16=True):
    W1, b1, W2, b2, W3, b3 = unpack(p, nin, H, nout)
    r = to_bf16 if bf16 else (lambda a: np.asarray(a, np.float64))
    xq = r(x)
    z1 = xq @ r(W1).T + b1
    a1 = r(silu(z1))
    z2 = a1 @ r(W2).T + b2
    a2 = r(silu(z2))
    y = a2 @ r(W3).T + b3
    return dict(x=xq, z1=z1, a1=a1, z2=z2, a2=a2, y=y, W2=r(W2), W3=r(W3))


def mixture_nll(y, tgt, K, D):
    """Per-sample NLL and d(mean NLL)/dy."""
    B = y.shape[0]
    logits = y[:, :K]
    mu = y[:, K:K + K * D].reshape(B, K, D)
    raw = y[:, K + K * D:].reshape(B, K, D)
    ls = np.clip(raw, -7.0, 5.0)
    lw = logits - np.logaddexp.reduce(logits, axis=1, keepdims=True)
    diff = tgt[:, None, :] - mu
    lp = lw + (-LOG2PI_HALF * D) + np.sum(-0.5 * (diff * np.exp(-ls)) ** 2 - ls, axis=2)
    ll = np.logaddexp.reduce(lp, axis=1)
    r = np.exp(lp - ll[:, None])
    w = np.exp(lw)
    g = np.zeros_like(y)
    g[:, :K] = (w - r) / B
    iv = np.exp(-2.0 * ls)
    g[:, K:K + K * D] = (-(r[:, :, None]) * diff * iv).reshape(B, K * D) / B
    gls = -(r[:, :, None]) * (diff * diff * iv - 1.0)
    gls = np.where((raw > -7.0) & (raw < 5.0), gls, 0.0)
    g[:, K + K * D:] = gls.reshape(B, K * D) / B
    return -ll, g


def gradients(p, x, tgt, nin, H, K, D, bf16=True):
    nout = K + 2 * K * D
    f = forward(p, x, nin, H, nout, bf16)
    r = to_bf16 if bf16 else (lambda a: np.asarray(a, np.float64))
    loss, dy = mixture_nll(f["y"], np.asarray(tgt, np.float64), K, D)
    dW3 = r(dy).T @ f["a2"]
    db3 = dy.sum(0)
    d2 = (r(dy) @ f["W3"]) * dsilu(f["z2"])
    dW2 = r(d2).T @ f["a1"]
    db2 = d2.sum(0)
    d1 = (r(d2) @ f["W2"]) * dsilu(f["z1"])
    dW1 = r(d1).T @ f["x"]
    db1 = d1.sum(0)
    g = np.concatenate([dW1.ravel(), db1, dW2.ravel(), db2, dW3.ravel(), db3])
    return float(loss.mean()), g
