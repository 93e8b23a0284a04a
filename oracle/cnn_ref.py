"""CPU restatement (numpy) of the CU-pruning network's forward and backward passes.

Test infrastructure only: the GPU kernels (uavs3e_gb300/csrc/cnn.cu) are checked against it.
It rounds to bf16 at the same points as the GPU path (inputs, weights, ReLU outputs, logits
gradients, data gradients) and accumulates in float32, so the two agree to accumulation-order
differences.  Layout: activations NHWC, weights [Cout][Kp] with k = (ky * ks + kx) * Cin + ci.
"""
import numpy as np

# EXACT = True turns every rounding off and computes in float64 (finite-difference checks of
# the backward pass itself)
EXACT = False


def _dt():
    return np.float64 if EXACT else np.float32


def bf16(a):
    """round float32 to bfloat16 (nearest even) and return float32"""
    if EXACT:
        return np.asarray(a, dtype=np.float64)
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def im2col(x, ks, stride):
    """x [B][H][W][C] -> columns [B*Ho*Wo][ks*ks*C] (zero padding ks//2)"""
    B, H, W, C = x.shape
    p = ks // 2
    Ho, Wo = (H + 2 * p - ks) // stride + 1, (W + 2 * p - ks) // stride + 1
    xp = np.zeros((B, H + 2 * p, W + 2 * p, C), _dt())
    xp[:, p:p + H, p:p + W] = x
    cols = np.zeros((B, Ho, Wo, ks, ks, C), _dt())
    for ky in range(ks):
        for kx in range(ks):
            cols[:, :, :, ky, kx] = xp[:, ky:ky + stride * Ho:stride, kx:kx + stride * Wo:stride]
    return cols.reshape(B * Ho * Wo, ks * ks * C), (Ho, Wo)


def col2im(dcols, shape, ks, stride):
    """adjoint of im2col: [B*Ho*Wo][ks*ks*C] -> [B][H][W][C]"""
    B, H, W, C = shape
    p = ks // 2
    Ho, Wo = (H + 2 * p - ks) // stride + 1, (W + 2 * p - ks) // stride + 1
    d = dcols.reshape(B, Ho, Wo, ks, ks, C)
    xp = np.zeros((B, H + 2 * p, W + 2 * p, C), _dt())
    for ky in range(ks):
        for kx in range(ks):
            xp[:, ky:ky + stride * Ho:stride, kx:kx + stride * Wo:stride] += d[:, :, :, ky, kx]
    return xp[:, p:p + H, p:p + W]


def conv_fwd(x, w, b, ks, stride, relu, out_f32=False):
    cols, (Ho, Wo) = im2col(x, ks, stride)
    K = cols.shape[1]
    y = cols @ w[:, :K].T + b[None, :]
    if relu:
        y = np.maximum(y, 0)
    y = y.reshape(x.shape[0], Ho, Wo, -1).astype(_dt())
    return y if out_f32 else bf16(y)


def conv_bwd(dy, x, w, ks, stride, need_dx=True):
    """dy: gradient at the pre-activation output [B][Ho][Wo][Cout] (bf16 values); returns
    (dw [Cout][Kp], db [Cout], dx [B][H][W][Cin] masked by x > 0 and rounded to bf16)"""
    cols, _ = im2col(x, ks, stride)
    K = cols.shape[1]
    d2 = dy.reshape(-1, dy.shape[-1])
    dw = np.zeros_like(w, dtype=_dt())
    dw[:, :K] = d2.T @ cols
    db = d2.sum(0)
    dx = None
    if need_dx:
        dcols = d2 @ w[:, :K]
        dx = col2im(dcols, x.shape, ks, stride)
        dx = bf16(np.where(x > 0, dx, 0))
    return dw, db, dx


def head_loss(logits, labels):
    """logits [B][16][48] float32, labels [B][40] uint8 -> (loss parts [4], dlogits bf16)"""
    B = logits.shape[0]
    L = logits.astype(np.float64)
    g = np.zeros_like(L)
    lab = labels.astype(np.float64)

    def bce(s, y):
        return np.maximum(s, 0) - s * y + np.log1p(np.exp(-np.abs(s))), 1 / (1 + np.exp(-s)) - y

    s64 = L[:, :, 2].mean(1)
    l64, d = bce(s64, lab[:, 0])
    g[:, :, 2] += d[:, None] / 16
    cell = np.arange(16)
    quad = (cell // 4 // 2) * 2 + (cell % 4) // 2
    s32 = np.stack([L[:, quad == q, 1].mean(1) for q in range(4)], 1)
    l32, d = bce(s32, lab[:, 1:5])
    g[:, :, 1] += d[:, quad] / 4 / 4
    l16, d = bce(L[:, :, 0], lab[:, 5:21])
    g[:, :, 0] += d / 16
    z = L[:, :, 3:36]
    mx = z.max(2, keepdims=True)
    e = np.exp(z - mx)
    sm = e / e.sum(2, keepdims=True)
    ym = labels[:, 21:37].astype(int)
    lm = (np.log(e.sum(2)) + mx[:, :, 0] - np.take_along_axis(z, ym[:, :, None], 2)[:, :, 0])
    oh = np.zeros_like(sm)
    np.put_along_axis(oh, ym[:, :, None], 1.0, 2)
    g[:, :, 3:36] += (sm - oh) / 16
    loss = np.array([l64.mean(), l32.mean(1).mean(), l16.mean(1).mean(), lm.mean(1).mean()])
    return loss, bf16((g / B).astype(_dt()))


def forward(x0, params, layers, head):
    """activations of every layer (bf16 values) and the head logits (float32)"""
    acts = [x0]
    for (cin, cout, ks, st), (w, b) in zip(layers, params[:-1]):
        acts.append(conv_fwd(acts[-1], w, b, ks, st, True))
    w, b = params[-1]
    logits = conv_fwd(acts[-1], w, b, head[2], head[3], False, out_f32=True)
    return acts, logits.reshape(x0.shape[0], 16, -1)


def backward(acts, logits, labels, params, layers, head):
    loss, dlog = head_loss(logits, labels)
    grads = [None] * len(params)
    w, b = params[-1]
    dy = dlog.reshape(acts[-1].shape[0], 4, 4, -1)
    dw, db, dx = conv_bwd(dy, acts[-1], w, head[2], head[3])
    grads[-1] = (dw, db)
    for i in range(len(layers) - 1, -1, -1):
        cin, cout, ks, st = layers[i]
        w, b = params[i]
        dw, db, dxp = conv_bwd(dx, acts[i], w, ks, st, need_dx=i > 0)
        grads[i] = (dw, db)
        dx = dxp
    return loss, grads
