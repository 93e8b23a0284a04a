"""Learned CU-partition / intra-mode pruning beside the bit-exact lattice.

A small CNN sees a 64x64 luma CTU and a constant QP plane and predicts the quad-tree split
flags at the 64, 32 and 16 levels and an 8-mode intra shortlist per 16x16 cell.  Training data
are the decisions the plain path makes: the batched intra lattice (bit-exact costs) evaluated
on square CUs, an RD cost J = SSD + lambda * R per (CU, mode) with R estimated from the coded
levels, the best mode per CU and a bottom-up quad-tree comparison for the split flags.  The
pruned search keeps the full lattice as its fallback: a level is decided from the network only
when its probability is beyond the confidence threshold, and a CU's modes are cut to the
shortlist; everything else is searched as before.

The network's kernels (uavs3e_gb300/csrc/cnn.cu) are bf16 tensor-core implicit GEMMs with FP32
accumulation (forward, data and weight gradients), a loss kernel and Adam; this module owns the
device buffers (torch allocations) and drives them through the C ABI.
"""
import ctypes as C

import numpy as np

from . import check, lib

# (Cin, Cout, kernel, stride) of the four convolutions and the 1x1 head
LAYERS = [(2, 16, 3, 2), (16, 32, 3, 2), (32, 32, 3, 2), (32, 64, 3, 2)]
HEAD = (64, 48, 1, 1)
N_MODES = 33
SHORTLIST = 8
LAMBDA_QP = lambda qp: 0.57 * 2.0 ** ((qp - 12) / 3.0)  # noqa: E731


def kpad(cin, ks):
    return (ks * ks * cin + 15) // 16 * 16


def _declare(L):
    P, I, F = C.c_void_p, C.c_int, C.c_float
    L.uavs3e_cuda_cnn_conv_fwd.argtypes = [P, P, P, P, I, I, I, I, I, I, I, I, I, I, P]
    L.uavs3e_cuda_cnn_conv_dgrad.argtypes = [P, P, P, P, P, I, I, I, I, I, I, I, I, P]
    L.uavs3e_cuda_cnn_conv_wgrad.argtypes = [P, P, P, P, I, I, I, I, I, I, I, I, P]
    L.uavs3e_cuda_cnn_input.argtypes = [P, I, I, I, P, I, I, P, P]
    L.uavs3e_cuda_cnn_head_loss.argtypes = [P, P, I, P, P, P]
    L.uavs3e_cuda_cnn_adam.argtypes = [P, P, P, P, P, I, F, F, F, F, I, P]


def init_params(seed=0):
    """He-normal weights [Cout][Kp] (entries beyond K are 0) and zero biases, float32"""
    rng = np.random.default_rng(seed)
    out = []
    for cin, cout, ks, st in LAYERS + [HEAD]:
        K, Kp = ks * ks * cin, kpad(cin, ks)
        w = np.zeros((cout, Kp), np.float32)
        w[:, :K] = rng.normal(0.0, np.sqrt(2.0 / K), (cout, K)).astype(np.float32)
        if (cin, cout, ks, st) == HEAD:
            w *= 0.1
        out.append((w, np.zeros(cout, np.float32)))
    return out


class PruneNet:
    """the network on the GPU for batches of B CTUs (B a multiple of 1; rows are padded by the
    kernels' own shape rules: B * 16 output cells must be a multiple of 16, always true)"""

    def __init__(self, B, params=None, seed=0):
        import torch
        self.torch, self.B = torch, B
        self.L = lib()
        _declare(self.L)
        dev = "cuda"
        params = params or init_params(seed)
        self.shapes = []     # (B, Hin, Win, Cin, Cout, ks, stride, Kp, Hout)
        h = 64
        for cin, cout, ks, st in LAYERS + [HEAD]:
            ho = (h + 2 * (ks // 2) - ks) // st + 1
            self.shapes.append((h, cin, cout, ks, st, kpad(cin, ks), ho))
            h = ho
        self.w32 = [torch.from_numpy(w.copy()).to(dev) for w, _ in params]
        self.b32 = [torch.from_numpy(b.copy()).to(dev) for _, b in params]
        self.wbf = [w.to(torch.bfloat16) for w in self.w32]
        self.mw = [torch.zeros_like(w) for w in self.w32]
        self.vw = [torch.zeros_like(w) for w in self.w32]
        self.mb = [torch.zeros_like(b) for b in self.b32]
        self.vb = [torch.zeros_like(b) for b in self.b32]
        self.gw = [torch.zeros_like(w) for w in self.w32]
        self.gb = [torch.zeros_like(b) for b in self.b32]
        self.acts = [torch.zeros((B, 64, 64, 2), dtype=torch.bfloat16, device=dev)]
        for (h_in, cin, cout, ks, st, kp, ho) in self.shapes[:-1]:
            self.acts.append(torch.zeros((B, ho, ho, cout), dtype=torch.bfloat16, device=dev))
        self.logits = torch.zeros((B, 16, HEAD[1]), dtype=torch.float32, device=dev)
        self.dlog = torch.zeros((B, 16, HEAD[1]), dtype=torch.bfloat16, device=dev)
        self.dx = [torch.zeros_like(a) for a in self.acts]
        self.wt = torch.zeros(64 * 9 * 64, dtype=torch.bfloat16, device=dev)
        self.loss = torch.zeros(4, dtype=torch.float32, device=dev)
        self.step_no = 0

    def _stream(self):
        return self.torch.cuda.current_stream().cuda_stream

    def params(self):
        return [(w.cpu().numpy(), b.cpu().numpy()) for w, b in zip(self.w32, self.b32)]

    def load_input(self, d_pic, stride, W, H, d_ctu_xy, n, qp):
        check(self.L.uavs3e_cuda_cnn_input(d_pic, stride, W, H, d_ctu_xy, n, qp, self.acts[0].data_ptr(),
                                           self._stream()), "cnn_input")

    def forward(self):
        st = self._stream()
        for i, (h, cin, cout, ks, s, kp, ho) in enumerate(self.shapes):
            last = i == len(self.shapes) - 1
            y = self.logits if last else self.acts[i + 1]
            check(self.L.uavs3e_cuda_cnn_conv_fwd(self.acts[i].data_ptr(), self.wbf[i].data_ptr(),
                                                  self.b32[i].data_ptr(), y.data_ptr(), 1 if last else 0, self.B, h, h,
                                                  cin, cout, ks, s, kp, 0 if last else 1, st), "cnn_conv_fwd")
        return self.logits

    def backward(self, d_labels):
        st = self._stream()
        check(self.L.uavs3e_cuda_cnn_head_loss(self.logits.data_ptr(), d_labels.data_ptr(), self.B,
                                               self.dlog.data_ptr(), self.loss.data_ptr(), st), "cnn_head_loss")
        dy = self.dlog
        for i in range(len(self.shapes) - 1, -1, -1):
            h, cin, cout, ks, s, kp, ho = self.shapes[i]
            check(self.L.uavs3e_cuda_cnn_conv_wgrad(dy.data_ptr(), self.acts[i].data_ptr(), self.gw[i].data_ptr(),
                                                    self.gb[i].data_ptr(), self.B, h, h, cin, cout, ks, s, kp, st),
                  "cnn_conv_wgrad")
            if i > 0:
                check(self.L.uavs3e_cuda_cnn_conv_dgrad(dy.data_ptr(), self.wbf[i].data_ptr(), self.acts[i].data_ptr(),
                                                        self.dx[i].data_ptr(), self.wt.data_ptr(), self.B, h, h, cin,
                                                        cout, ks, s, kp, st), "cnn_conv_dgrad")
                dy = self.dx[i]
        return self.loss

    def adam(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        st = self._stream()
        self.step_no += 1
        for i in range(len(self.shapes)):
            check(self.L.uavs3e_cuda_cnn_adam(self.w32[i].data_ptr(), self.mw[i].data_ptr(), self.vw[i].data_ptr(),
                                              self.gw[i].data_ptr(), self.wbf[i].data_ptr(), self.w32[i].numel(), lr,
                                              b1, b2, eps, self.step_no, st), "cnn_adam")
            check(self.L.uavs3e_cuda_cnn_adam(self.b32[i].data_ptr(), self.mb[i].data_ptr(), self.vb[i].data_ptr(),
                                              self.gb[i].data_ptr(), None, self.b32[i].numel(), lr, b1, b2, eps,
                                              self.step_no, st), "cnn_adam")


# ----------------------------------------------------------------------------- labels

def square_cus(W, H):
    """square lattice CUs (8..64) of the full 64x64 CTUs of a W x H picture, by CTU"""
    from . import CU
    out = []
    for s in (64, 32, 16, 8):
        for y in range(0, H // 64 * 64, s):
            for x in range(0, W // 64 * 64, s):
                out.append((x, y, s, s))
    c = np.zeros(len(out), dtype=CU)
    arr = np.array(out, dtype=np.int32)
    c["x"], c["y"], c["w"], c["h"] = arr[:, 0], arr[:, 1], arr[:, 2], arr[:, 3]
    return c


def rd_costs(q, cus, qp, qi=0, n_qp=1):
    """J = SSD + lambda * R per (CU, mode) from the lattice's first-pass statistics at one QP;
    R = 1 bit for an all-zero block, else 4 + 1.5 bits per coded level + 1 bit per level unit"""
    rec = q.reshape(len(cus), N_MODES, n_qp)[:, :, qi]
    nz = rec["num_nz"].astype(np.float64)
    bits = np.where(nz > 0, 4.0 + 1.5 * nz + rec["sum_abs"].astype(np.float64), 1.0)
    return rec["ssd"].astype(np.float64) + LAMBDA_QP(qp) * bits


def plain_decisions(J, cus, W, H):
    """quad-tree decisions of the plain path for every full CTU: labels [n_ctu][40] (u8) with
    [0] split64, [1..4] split32 (quadrants raster), [5..20] split16 (cells raster), [21..36] the
    best mode of each 16x16 cell, and the CTU origins [n_ctu][2]"""
    best = J.min(1)
    arg = J.argmin(1)
    idx = {(int(c["x"]), int(c["y"]), int(c["w"])): i for i, c in enumerate(cus)}
    cw, ch = W // 64, H // 64
    labels = np.zeros((cw * ch, 40), np.uint8)
    xy = np.zeros((cw * ch, 2), np.int32)
    split_bits = LAMBDA_QP(32) * 1.0

    def node(x, y, s):
        own = best[idx[(x, y, s)]] + split_bits
        if s == 8:
            return own, False
        h = s // 2
        kids = sum(node(x + dx, y + dy, h)[0] for dy in (0, h) for dx in (0, h)) + split_bits
        return min(own, kids), kids < own

    for cy in range(ch):
        for cx in range(cw):
            b = cy * cw + cx
            x0, y0 = cx * 64, cy * 64
            xy[b] = (x0, y0)
            labels[b, 0] = node(x0, y0, 64)[1]
            for qd in range(4):
                labels[b, 1 + qd] = node(x0 + 32 * (qd & 1), y0 + 32 * (qd >> 1), 32)[1]
            for c in range(16):
                x, y = x0 + 16 * (c % 4), y0 + 16 * (c // 4)
                labels[b, 5 + c] = node(x, y, 16)[1]
                labels[b, 21 + c] = arg[idx[(x, y, 16)]]
    return labels, xy
