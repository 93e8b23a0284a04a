"""CPU: the pruning network's numpy restatement (the GPU kernels' checker) and the plain-path
decision labels."""
import numpy as np

import cnn_ref
from uavs3e_gb300 import cnn


def tiny_net(seed=0, B=2):
    rng = np.random.default_rng(seed)
    params = cnn.init_params(seed)
    params = [(w.astype(np.float64), rng.normal(0, 0.1, b.shape)) for w, b in params]
    x0 = rng.normal(0, 1, (B, 64, 64, 2))
    labels = np.zeros((B, 40), np.uint8)
    labels[:, :21] = rng.integers(0, 2, (B, 21))
    labels[:, 21:37] = rng.integers(0, 33, (B, 16))
    return params, x0, labels


def total_loss(params, x0, labels):
    acts, logits = cnn_ref.forward(x0, params, cnn.LAYERS, cnn.HEAD)
    loss, _ = cnn_ref.head_loss(logits, labels)
    return loss.sum()


def test_backward_matches_finite_differences():
    cnn_ref.EXACT = True
    try:
        params, x0, labels = tiny_net()
        acts, logits = cnn_ref.forward(x0, params, cnn.LAYERS, cnn.HEAD)
        _, grads = cnn_ref.backward(acts, logits, labels, params, cnn.LAYERS, cnn.HEAD)
        rng = np.random.default_rng(3)
        eps = 1e-5
        for li in range(len(params)):
            w, b = params[li]
            K = cnn.LAYERS[li][2] ** 2 * cnn.LAYERS[li][0] if li < 4 else cnn.HEAD[0]
            for _ in range(3):
                o, k = rng.integers(0, w.shape[0]), rng.integers(0, K)
                w[o, k] += eps
                up = total_loss(params, x0, labels)
                w[o, k] -= 2 * eps
                dn = total_loss(params, x0, labels)
                w[o, k] += eps
                num = (up - dn) / (2 * eps)
                assert abs(num - grads[li][0][o, k]) <= 1e-6 + 1e-4 * abs(num), (li, o, k, num, grads[li][0][o, k])
            o = rng.integers(0, b.shape[0])
            b[o] += eps
            up = total_loss(params, x0, labels)
            b[o] -= 2 * eps
            dn = total_loss(params, x0, labels)
            b[o] += eps
            num = (up - dn) / (2 * eps)
            assert abs(num - grads[li][1][o]) <= 1e-6 + 1e-4 * abs(num)
    finally:
        cnn_ref.EXACT = False


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.00390625, 1.005859375, 1.0078125, -3.14159, 0.0], np.float32)
    r = cnn_ref.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125 and r[3] == 1.0078125
    assert abs(r[4] + 3.140625) < 1e-7 and r[5] == 0.0


def test_plain_decisions_quad_tree():
    W, H = 128, 64
    cus = cnn.square_cus(W, H)
    J = np.full((len(cus), 33), 1e6)
    # CTU 0: cheap 8x8 CUs everywhere (split to 8); CTU 1: cheap 64x64 with mode 7 (no split)
    for i, c in enumerate(cus):
        if c["x"] < 64:
            if c["w"] == 8:
                J[i, 3] = 10.0
        else:
            if c["w"] == 64:
                J[i, 7] = 10.0
            if c["w"] == 16:
                J[i, 5] = 1e5
    labels, xy = cnn.plain_decisions(J, cus, W, H)
    assert xy.tolist() == [[0, 0], [64, 0]]
    assert labels[0, 0] == 1 and labels[0, 1:5].all() and labels[0, 5:21].all()
    assert labels[1, 0] == 0
    assert (labels[1, 21:37] == 5).all()


def test_bd_rate_of_known_curves():
    rate = np.array([1000.0, 1800.0, 3100.0, 5200.0])
    psnr = np.array([31.0, 33.5, 36.0, 38.4])
    assert abs(cnn.bd_rate(rate, psnr, rate, psnr)) < 1e-9
    # the same curve at 1.1x the rate everywhere: +10 %; at 0.95x: -5 %
    assert abs(cnn.bd_rate(rate, psnr, 1.1 * rate, psnr) - 10.0) < 1e-6
    assert abs(cnn.bd_rate(rate, psnr, 0.95 * rate, psnr) + 5.0) < 1e-6
    # a curve that needs more PSNR-matched rate is worse (positive)
    assert cnn.bd_rate(rate, psnr, rate, psnr - 0.5) > 0


def test_search_rd_full_and_keep_everything_agree():
    W, H = 128, 64
    cus = cnn.square_cus(W, H)
    rng = np.random.default_rng(3)
    S = rng.uniform(100, 5000, (len(cus), 33)) * (cus["w"].astype(float)[:, None] / 8) ** 2
    R = rng.uniform(1, 200, (len(cus), 33))
    qp = 37
    J = S + cnn.LAMBDA_QP(qp) * R
    labels, xy = cnn.plain_decisions(J, cus, W, H, qp)
    full = cnn.search_rd(J, S, R, cus, xy, None, 0.9, qp)
    n = len(xy)
    keep_all = (np.full(n, 0.5), np.full((n, 4), 0.5), np.full((n, 16), 0.5), np.tile(np.arange(8), (n, 16, 1)))
    same = cnn.search_rd(J, S, R, cus, xy, keep_all, 0.9, qp, shortlist=False)
    assert np.allclose(full, same)
    assert abs(full[2] - 1.0) < 1e-12
    # the chosen decisions' J equals the quad-tree minimum of plain_decisions' recursion
    jf = full[0] + cnn.LAMBDA_QP(qp) * full[1]
    idx = {(int(c["x"]), int(c["y"]), int(c["w"])): i for i, c in enumerate(cus)}
    lam = cnn.LAMBDA_QP(qp)

    def best(x, y, s):
        own = J[idx[(x, y, s)]].min() + lam
        if s == 8:
            return own
        h = s // 2
        return min(own, sum(best(x + dx, y + dy, h) for dy in (0, h) for dx in (0, h)) + lam)
    assert abs(jf - sum(best(int(x), int(y), 64) for x, y in xy)) < 1e-6 * jf
    # a shortlist that misses the best modes cannot lower the rate-distortion cost
    worst = (np.full(n, 0.5), np.full((n, 4), 0.5), np.full((n, 16), 0.5),
             np.tile(np.argsort(-J.mean(0))[:8], (n, 16, 1)))
    pr = cnn.search_rd(J, S, R, cus, xy, worst, 0.9, qp)
    assert pr[0] + lam * pr[1] >= jf - 1e-6 * jf and pr[2] < 1.0


def test_encoder_label_fixture_and_derivation():
    """the committed labels from the reference encoder's CU decisions: shapes, value ranges, and
    the derivation on a hand-made CU list"""
    import os
    import sys
    golden = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    sys.path.insert(0, golden)
    import make_encoder_labels as mel
    d = np.load(os.path.join(golden, "encoder_labels.npz"))
    lab = d["labels"]
    assert lab.shape == (len(d["seeds"]), len(d["qps"]), (int(d["width"]) // 64) * (int(d["height"]) // 64), 40)
    assert lab[..., :21].max() <= 1 and lab[..., 21:37].max() <= 32
    # an unsplit CTU implies unsplit quadrants and cells
    whole = lab[..., 0] == 0
    assert not lab[whole][:, 1:21].any()
    # a 128x64 picture: CTU 0 one 64x64 CU (mode 7); CTU 1 four 32x32 CUs, the first split into
    # 16x16 CUs (modes 3), the others 32x32 (mode 12)
    cus = [(0, 0, 64, 64, 1, 7)]
    for q in range(4):
        x, y = 64 + 32 * (q & 1), 32 * (q >> 1)
        if q == 0:
            cus += [(x + 16 * (k & 1), y + 16 * (k >> 1), 16, 16, 1, 3) for k in range(4)]
        else:
            cus.append((x, y, 32, 32, 1, 12))
    labels, xy = mel.ctu_labels(np.array(cus), 128, 64)
    assert xy.tolist() == [[0, 0], [64, 0]]
    assert labels[0, 0] == 0 and not labels[0, 1:21].any() and (labels[0, 21:37] == 7).all()
    assert labels[1, 0] == 1 and labels[1, 1:5].tolist() == [1, 0, 0, 0]
    assert not labels[1, 5:21].any()
    assert labels[1, 21] == 3 and labels[1, 23] == 12
