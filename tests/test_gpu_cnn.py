"""GPU: the pruning network's bf16 tensor-core kernels against the numpy restatement, and a
short training run that must beat the prior."""
import numpy as np
import pytest

import cnn_ref

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-12)


def setup_net(gpu, B, seed):
    import torch
    from uavs3e_gb300 import cnn
    rng = np.random.default_rng(seed)
    params = cnn.init_params(seed)
    params = [(w, rng.normal(0, 0.05, b.shape).astype(np.float32)) for w, b in params]
    net = cnn.PruneNet(B, params=params)
    x0 = cnn_ref.bf16(rng.normal(0, 1, (B, 64, 64, 2)).astype(np.float32))
    net.acts[0].copy_(torch.from_numpy(x0).to(torch.bfloat16))
    labels = np.zeros((B, 40), np.uint8)
    labels[:, :21] = rng.integers(0, 2, (B, 21))
    labels[:, 21:37] = rng.integers(0, 33, (B, 16))
    ref_params = [(cnn_ref.bf16(w), b) for w, b in params]
    return net, x0, labels, ref_params


@pytest.mark.parametrize("B,seed", [(4, 1), (7, 2)])
def test_forward_backward_match_oracle(gpu, B, seed):
    import torch
    from uavs3e_gb300 import cnn
    net, x0, labels, ref_params = setup_net(gpu, B, seed)
    logits = net.forward()
    d_lab = torch.from_numpy(labels).cuda()
    loss = net.backward(d_lab)
    torch.cuda.synchronize()
    acts, ref_logits = cnn_ref.forward(x0, ref_params, cnn.LAYERS, cnn.HEAD)
    for i in range(1, len(acts)):
        assert rel(net.acts[i].float().cpu().numpy(), acts[i]) < 1e-2, f"activation {i}"
    assert rel(logits.cpu().numpy(), ref_logits) < 1e-2
    # gradients from the oracle fed with the GPU's own activations and logits, so the check
    # isolates the backward kernels
    gpu_acts = [x0] + [net.acts[i].float().cpu().numpy() for i in range(1, len(acts))]
    ref_loss, grads = cnn_ref.backward(gpu_acts, logits.cpu().numpy(), labels, ref_params, cnn.LAYERS, cnn.HEAD)
    assert np.allclose(loss.cpu().numpy(), ref_loss, rtol=1e-4, atol=1e-5)
    for i, (dw, db) in enumerate(grads):
        assert rel(net.gw[i].cpu().numpy(), dw) < 2e-2, f"weight gradient {i}"
        assert rel(net.gb[i].cpu().numpy(), db) < 2e-2, f"bias gradient {i}"
    # every tensor-core tile completed its MMAs within the bounded wait
    assert gpu.lib().uavs3e_cuda_cnn_timeouts() == 0


def test_adam_step_matches_formula(gpu):
    import torch
    from uavs3e_gb300 import cnn
    net, x0, labels, _ = setup_net(gpu, 4, 3)
    net.forward()
    net.backward(torch.from_numpy(labels).cuda())
    w0 = [w.cpu().numpy().copy() for w in net.w32]
    g = [x.cpu().numpy().copy() for x in net.gw]
    net.adam(lr=1e-3)
    torch.cuda.synchronize()
    for i in range(len(w0)):
        # first step: m = 0.1 g, v = 0.001 g^2, corrections 0.1 and 0.001 -> w - lr g / (|g| + eps)
        want = w0[i] - 1e-3 * g[i] / (np.abs(g[i]) + 1e-8)
        assert np.allclose(net.w32[i].cpu().numpy(), want, rtol=1e-4, atol=1e-6)
        assert np.array_equal(net.wbf[i].float().cpu().numpy(),
                              cnn_ref.bf16(net.w32[i].cpu().numpy()))


def learnable_batch(rng, B):
    """CTUs of stripes at a random angle and contrast: split flags from the contrast of the
    quadrant / cell, the mode label from the stripe angle (a function the network can learn)"""
    yy, xx = np.mgrid[0:64, 0:64]
    x0 = np.zeros((B, 64, 64, 2), np.float32)
    labels = np.zeros((B, 40), np.uint8)
    for b in range(B):
        ang = rng.integers(0, 8)
        th = np.pi * ang / 8
        amp = rng.uniform(0, 1, (4, 4))
        amp = np.kron(amp, np.ones((16, 16)))
        img = amp * np.sin((xx * np.cos(th) + yy * np.sin(th)) * 0.6)
        x0[b, :, :, 0] = img
        labels[b, 0] = amp.mean() > 0.5
        for q in range(4):
            labels[b, 1 + q] = amp[32 * (q >> 1):32 * (q >> 1) + 32, 32 * (q & 1):32 * (q & 1) + 32].mean() > 0.5
        for c in range(16):
            labels[b, 5 + c] = amp[16 * (c // 4), 16 * (c % 4)] > 0.5
            labels[b, 21 + c] = 3 + 4 * ang
    return cnn_ref.bf16(x0), labels


def test_training_learns_a_learnable_target(gpu):
    import torch
    from uavs3e_gb300 import cnn
    B = 32
    rng = np.random.default_rng(0)
    net = cnn.PruneNet(B, seed=5)
    first = None
    for it in range(150):
        x0, labels = learnable_batch(rng, B)
        net.acts[0].copy_(torch.from_numpy(x0).to(torch.bfloat16))
        net.forward()
        loss = net.backward(torch.from_numpy(labels).cuda()).sum().item()
        net.adam(lr=3e-3)
        first = loss if first is None else first
    x0, labels = learnable_batch(np.random.default_rng(99), B)
    net.acts[0].copy_(torch.from_numpy(x0).to(torch.bfloat16))
    logits = net.forward().cpu().numpy()
    assert loss < 0.6 * first
    pred16 = logits[:, :, 0] > 0
    acc16 = (pred16 == labels[:, 5:21].astype(bool)).mean()
    prior16 = max(labels[:, 5:21].mean(), 1 - labels[:, 5:21].mean())
    assert acc16 > prior16 + 0.1
    top8 = np.argsort(-logits[:, :, 3:36], axis=2)[:, :, :cnn.SHORTLIST]
    recall = (top8 == labels[:, 21:37, None]).any(2).mean()
    assert recall > 0.9


def test_pruning_beats_the_method_without_the_network(gpu):
    # trained on the plain path's decisions (lattice costs) of a few frames, evaluated on a
    # held-out frame: better mode shortlist than the prior and a cheaper pruned search
    from uavs3e_gb300 import cnn
    r = cnn.experiment(train_seeds=range(200, 203), test_seeds=(950,), steps=500, batch=64, taus=(0.9,),
                       width=640, height=384)
    assert r["loss_last"] < 0.6 * r["loss_first"]
    assert r["net"]["mode_top8_recall"] > r["prior"]["mode_top8_recall"] + 0.2
    net, prior = r["net"]["tau0.9"], r["prior"]["tau0.9"]
    assert net["rd_cost_increase"] < prior["rd_cost_increase"]
    assert net["work_fraction"] < 0.5
    assert r["pruned_lattice_tau0.9"]["speedup"] > 1.5


def test_network_learns_the_reference_encoders_decisions(gpu):
    # trained on the reference encoder's own final CUs (committed fixture of seeded 512x256
    # I-frames at 4 QPs), evaluated on its held-out frames: a better mode shortlist and 64x64
    # split decision than the method without the network
    import os
    from uavs3e_gb300 import cnn
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "encoder_labels.npz")
    r = cnn.encoder_label_experiment(path, steps=800, batch=64)
    assert r["loss_last"] < 0.6 * r["loss_first"]
    assert r["net"]["mode_top8_recall"] > r["prior"]["mode_top8_recall"] + 0.1
    assert r["net"]["split64_acc"] >= r["prior"]["split64_acc"]
    assert 0.0 < r["rd_model_agreement"]["split64"] <= 1.0


# single convolutions through the C ABI: stride 1 and 2, odd picture sizes (the data gradient's
# phase classes then differ in size), 8-channel groups and channel counts that are not a
# multiple of 8 (the element-wise gathers)
CONV_SHAPES = [  # B, H, Cin, Cout, ks, stride
    (16, 9, 16, 32, 3, 2),
    (4, 12, 32, 16, 3, 1),
    (16, 8, 8, 16, 3, 2),
    (16, 10, 6, 16, 3, 2),
    (16, 7, 2, 16, 3, 1),
    (4, 4, 64, 48, 1, 1),
    (4, 8, 16, 32, 1, 2),      # 1x1 at stride 2: three phase classes reach no tap (dx = 0 there)
]


@pytest.mark.parametrize("B,H,Cin,Cout,ks,stride", CONV_SHAPES)
def test_conv_layer_matches_oracle(gpu, B, H, Cin, Cout, ks, stride):
    import torch
    from uavs3e_gb300 import cnn
    L = gpu.lib()
    cnn._declare(L)
    rng = np.random.default_rng(B * 1000 + H * 10 + Cin + stride)
    Kp = cnn.kpad(Cin, ks)
    K = ks * ks * Cin
    Ho = (H + 2 * (ks // 2) - ks) // stride + 1
    # a ReLU output: about a third of the inputs are 0 (the data gradient's mask)
    x = cnn_ref.bf16(np.maximum(rng.normal(0.2, 1, (B, H, H, Cin)), 0).astype(np.float32))
    w = np.zeros((Cout, Kp), np.float32)
    w[:, :K] = cnn_ref.bf16(rng.normal(0, 0.3, (Cout, K)).astype(np.float32))
    b = rng.normal(0, 0.1, Cout).astype(np.float32)
    dy = cnn_ref.bf16(rng.normal(0, 1, (B, Ho, Ho, Cout)).astype(np.float32))
    dev = lambda a, dt=torch.bfloat16: torch.from_numpy(np.ascontiguousarray(a)).to(dt).cuda()  # noqa: E731
    d_x, d_w, d_b, d_dy = dev(x), dev(w), dev(b, torch.float32), dev(dy)
    d_y = torch.zeros((B, Ho, Ho, Cout), dtype=torch.bfloat16, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    assert L.uavs3e_cuda_cnn_conv_fwd(d_x.data_ptr(), d_w.data_ptr(), d_b.data_ptr(), d_y.data_ptr(), 0, B, H, H,
                                      Cin, Cout, ks, stride, Kp, 1, st) == 0
    d_dw = torch.zeros((Cout, Kp), dtype=torch.float32, device="cuda")
    d_db = torch.zeros(Cout, dtype=torch.float32, device="cuda")
    assert L.uavs3e_cuda_cnn_conv_wgrad(d_dy.data_ptr(), d_x.data_ptr(), d_dw.data_ptr(), d_db.data_ptr(), B, H, H,
                                        Cin, Cout, ks, stride, Kp, st) == 0
    need_dx = Cin % 16 == 0
    if need_dx:
        d_dx = torch.zeros((B, H, H, Cin), dtype=torch.bfloat16, device="cuda")
        assert L.uavs3e_cuda_cnn_conv_dgrad(d_dy.data_ptr(), d_w.data_ptr(), d_x.data_ptr(), d_dx.data_ptr(),
                                            None, B, H, H, Cin, Cout, ks, stride, Kp, st) == 0
    torch.cuda.synchronize()
    y_ref = cnn_ref.conv_fwd(x, w, b, ks, stride, relu=True)
    dw_ref, db_ref, dx_ref = cnn_ref.conv_bwd(dy, x, w, ks, stride, need_dx=need_dx)
    assert rel(d_y.float().cpu().numpy(), y_ref) < 1e-2
    assert rel(d_dw.cpu().numpy(), dw_ref) < 1e-4
    assert rel(d_db.cpu().numpy(), db_ref) < 1e-4
    if need_dx:
        assert rel(d_dx.float().cpu().numpy(), dx_ref) < 1e-2
    assert L.uavs3e_cuda_cnn_timeouts() == 0


def test_conv_rejects_bad_shapes_and_alignment(gpu):
    """shapes outside the kernels' rules and tensors off a 16-byte boundary are refused before
    any launch"""
    import torch
    from uavs3e_gb300 import cnn
    L = gpu.lib()
    cnn._declare(L)
    B, H, Cin, Cout, ks = 16, 8, 16, 32, 3
    Kp = cnn.kpad(Cin, ks)
    x = torch.zeros(B * H * H * Cin + 8, dtype=torch.bfloat16, device="cuda")
    w = torch.zeros(Cout * Kp, dtype=torch.bfloat16, device="cuda")
    b = torch.zeros(Cout, dtype=torch.float32, device="cuda")
    y = torch.zeros(B * H * H * Cout, dtype=torch.bfloat16, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    ok = L.uavs3e_cuda_cnn_conv_fwd(x.data_ptr(), w.data_ptr(), b.data_ptr(), y.data_ptr(), 0, B, H, H, Cin, Cout,
                                    ks, 2, Kp, 1, st)
    assert ok == 0
    # stride 3
    assert L.uavs3e_cuda_cnn_conv_fwd(x.data_ptr(), w.data_ptr(), b.data_ptr(), y.data_ptr(), 0, B, H, H, Cin, Cout,
                                      ks, 3, Kp, 1, st) != 0
    # activations 2 bytes past a 16-byte boundary
    assert L.uavs3e_cuda_cnn_conv_fwd(x.data_ptr() + 2, w.data_ptr(), b.data_ptr(), y.data_ptr(), 0, B, H, H, Cin,
                                      Cout, ks, 2, Kp, 1, st) != 0
    dw = torch.zeros(Cout * Kp, dtype=torch.float32, device="cuda")
    assert L.uavs3e_cuda_cnn_conv_wgrad(y.data_ptr(), x.data_ptr() + 2, dw.data_ptr(), b.data_ptr(), B, H, H, Cin,
                                        Cout, ks, 2, Kp, st) != 0
    # data gradient: output channels not a multiple of 16
    assert L.uavs3e_cuda_cnn_conv_dgrad(y.data_ptr(), w.data_ptr(), x.data_ptr(), x.data_ptr(), None, B, H, H, Cin,
                                        24, ks, 2, Kp, st) != 0
    torch.cuda.synchronize()
