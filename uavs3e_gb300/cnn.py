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
# the encoder's rate-distortion lambda for an 8-bit QP (src/uavs3e.c:834)
LAMBDA_QP = lambda qp: 1.43631 * 2.0 ** ((qp - 16) / 4.0)  # noqa: E731


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
        # every layer's weights and biases are views of one flat FP32 buffer (and its moments,
        # gradients and bf16 copy), so one Adam launch updates them all; each view starts on a
        # multiple of 16 elements (Cout * Kp and Cout are), as the 16-byte gathers need
        sizes = []
        for w, b in params:
            sizes += [w.size, b.size]
        n = sum(sizes)
        self.flat32 = torch.zeros(n, dtype=torch.float32, device=dev)
        self.flat_m = torch.zeros_like(self.flat32)
        self.flat_v = torch.zeros_like(self.flat32)
        self.flat_g = torch.zeros_like(self.flat32)
        self.flat_bf = torch.zeros(n, dtype=torch.bfloat16, device=dev)

        def views(flat):
            out, off = [], 0
            for w, b in params:
                out.append(flat[off:off + w.size].view(w.shape))
                off += w.size
                out.append(flat[off:off + b.size].view(b.shape))
                off += b.size
            return out[0::2], out[1::2]

        self.w32, self.b32 = views(self.flat32)
        for (w, b), dw, db in zip(params, self.w32, self.b32):
            dw.copy_(torch.from_numpy(np.ascontiguousarray(w, np.float32)))
            db.copy_(torch.from_numpy(np.ascontiguousarray(b, np.float32)))
        self.flat_bf.copy_(self.flat32.to(torch.bfloat16))
        self.wbf, _ = views(self.flat_bf)
        self.gw, self.gb = views(self.flat_g)
        self.acts = [torch.zeros((B, 64, 64, 2), dtype=torch.bfloat16, device=dev)]
        for (h_in, cin, cout, ks, st, kp, ho) in self.shapes[:-1]:
            self.acts.append(torch.zeros((B, ho, ho, cout), dtype=torch.bfloat16, device=dev))
        self.logits = torch.zeros((B, 16, HEAD[1]), dtype=torch.float32, device=dev)
        self.dlog = torch.zeros((B, 16, HEAD[1]), dtype=torch.bfloat16, device=dev)
        self.dx = [torch.zeros_like(a) for a in self.acts]
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
                                                        self.dx[i].data_ptr(), None, self.B, h, h, cin,
                                                        cout, ks, s, kp, st), "cnn_conv_dgrad")
                dy = self.dx[i]
        return self.loss

    def adam(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        st = self._stream()
        self.step_no += 1
        # every weight and bias in one launch (the biases' bf16 copies are written but not read)
        check(self.L.uavs3e_cuda_cnn_adam(self.flat32.data_ptr(), self.flat_m.data_ptr(), self.flat_v.data_ptr(),
                                          self.flat_g.data_ptr(), self.flat_bf.data_ptr(), self.flat32.numel(), lr,
                                          b1, b2, eps, self.step_no, st), "cnn_adam")


def step_flops(B):
    """tensor multiply-adds x 2 of one training step at batch B: every convolution's forward GEMM,
    its weight-gradient GEMM, and the data-gradient GEMM of every layer but the first (real K,
    without the padding to 16)"""
    tot, h = 0, 64
    for i, (cin, cout, ks, st) in enumerate(LAYERS + [HEAD]):
        ho = (h + 2 * (ks // 2) - ks) // st + 1
        gemm = 2.0 * B * ho * ho * cout * ks * ks * cin
        tot += gemm * (3 if i > 0 else 2)
        h = ho
    return tot


def step_time(B=1024, reps=20, seed=0):
    """milliseconds of one training step (forward, head loss, backward, Adam) at batch B, CUDA
    events on the launching stream over `reps` steps after two warm-up steps; returns (ms, flops)"""
    import torch
    rng = np.random.default_rng(seed)
    net = PruneNet(B, seed=seed)
    net.acts[0].copy_(torch.from_numpy(rng.normal(0, 1, (B, 64, 64, 2)).astype(np.float32)).to(torch.bfloat16))
    labels = np.zeros((B, 40), np.uint8)
    labels[:, :21] = rng.integers(0, 2, (B, 21))
    labels[:, 21:37] = rng.integers(0, 33, (B, 16))
    d_lab = torch.from_numpy(labels).cuda()

    def step():
        net.forward()
        net.backward(d_lab)
        net.adam()

    for _ in range(2):
        step()
    st = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(st)
    for _ in range(reps):
        step()
    e1.record(st)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps, step_flops(B)


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


def rd_terms(q, cus, qp, qi=0, n_qp=1):
    """(J, SSD, R) per (CU, mode) from the lattice's first-pass statistics at one QP: J = SSD +
    lambda R, R = 1 bit for an all-zero block, else 4 + 1.5 bits per coded level + 1 bit per
    level unit"""
    rec = q.reshape(len(cus), N_MODES, n_qp)[:, :, qi]
    nz = rec["num_nz"].astype(np.float64)
    bits = np.where(nz > 0, 4.0 + 1.5 * nz + rec["sum_abs"].astype(np.float64), 1.0)
    ssd = rec["ssd"].astype(np.float64)
    return ssd + LAMBDA_QP(qp) * bits, ssd, bits


def rd_costs(q, cus, qp, qi=0, n_qp=1):
    """J = SSD + lambda * R per (CU, mode) (rd_terms)"""
    return rd_terms(q, cus, qp, qi, n_qp)[0]


def plain_decisions(J, cus, W, H, qp=32):
    """quad-tree decisions of the plain path for every full CTU: labels [n_ctu][40] (u8) with
    [0] split64, [1..4] split32 (quadrants raster), [5..20] split16 (cells raster), [21..36] the
    best mode of each 16x16 cell, and the CTU origins [n_ctu][2]"""
    best = J.min(1)
    arg = J.argmin(1)
    idx = {(int(c["x"]), int(c["y"]), int(c["w"])): i for i, c in enumerate(cus)}
    cw, ch = W // 64, H // 64
    labels = np.zeros((cw * ch, 40), np.uint8)
    xy = np.zeros((cw * ch, 2), np.int32)
    split_bits = LAMBDA_QP(qp) * 1.0

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


# ----------------------------------------------------------------------------- data, training

def frame_dataset(frame, qp=32):
    """labels of the plain path for every full CTU of a frame (GPU lattice on the square CUs,
    org as the reconstructed neighbours) -> (ctus [n][64][64] u8, labels, xy, J, cus)"""
    d = frame_dataset_qps(frame, (qp,))[qp]
    return d[0], d[1], d[2], d[3], d[6]


def frame_dataset_qps(frame, qps):
    """frame_dataset at several QPs from one lattice run: {qp: (ctus, labels, xy, J, SSD, R, cus)}"""
    from . import intra_lattice
    H, W = frame.shape
    cus = square_cus(W, H)
    _, q = intra_lattice(frame, frame, cus, qps=tuple(qps), ipf=0)
    out = {}
    ctus = None
    for qi, qp in enumerate(qps):
        J, S, R = rd_terms(q, cus, qp, qi, len(qps))
        labels, xy = plain_decisions(J, cus, W, H, qp)
        if ctus is None:
            ctus = np.stack([frame[y:y + 64, x:x + 64] for x, y in xy])
        out[qp] = (ctus, labels, xy, J, S, R, cus)
    return out


def host_input(ctus, qp):
    """network input of CTUs (host): [n][64][64][2] float32, rounded to bf16 on upload; qp is one
    QP or one per CTU"""
    x = np.empty(ctus.shape + (2,), np.float32)
    x[..., 0] = (ctus.astype(np.float32) - 128.0) / 64.0
    q = np.asarray(qp, np.float32)
    x[..., 1] = ((q.reshape(-1, 1, 1) if q.ndim else q) - 32.0) / 8.0
    return x


def train(net, ctus, labels, qp=32, steps=300, lr=2e-3, seed=0):
    """Adam on random batches of net.B CTUs (qp: one QP or one per CTU); returns the loss (sum of
    the 4 parts) per step"""
    import torch
    rng = np.random.default_rng(seed)
    hist = []
    d_lab = torch.empty((net.B, 40), dtype=torch.uint8, device="cuda")
    qa = np.asarray(qp)
    for _ in range(steps):
        idx = rng.integers(0, len(ctus), net.B)
        net.acts[0].copy_(torch.from_numpy(host_input(ctus[idx], qa[idx] if qa.ndim else qa)).to(torch.bfloat16))
        d_lab.copy_(torch.from_numpy(labels[idx]))
        net.forward()
        hist.append(net.backward(d_lab).sum())
        net.adam(lr=lr)
    return [float(h) for h in torch.stack(hist).cpu()]


def predict(net, ctus, qp=32):
    """(split probabilities p64 [n], p32 [n][4], p16 [n][16], mode shortlist [n][16][8]) of CTUs"""
    import torch
    n = len(ctus)
    p64, p32, p16, top = [], [], [], []
    for s in range(0, n, net.B):
        part = ctus[s:s + net.B]
        x = np.zeros((net.B, 64, 64), np.uint8)
        x[:len(part)] = part
        net.acts[0].copy_(torch.from_numpy(host_input(x, qp)).to(torch.bfloat16))
        lg = net.forward().cpu().numpy()[:len(part)]
        sig = lambda v: 1.0 / (1.0 + np.exp(-v))  # noqa: E731
        p64.append(sig(lg[:, :, 2].mean(1)))
        cell = np.arange(16)
        quad = (cell // 8) * 2 + (cell % 4) // 2
        p32.append(sig(np.stack([lg[:, quad == qd, 1].mean(1) for qd in range(4)], 1)))
        p16.append(sig(lg[:, :, 0]))
        top.append(np.argsort(-lg[:, :, 3:36], axis=2)[:, :, :SHORTLIST])
    return np.concatenate(p64), np.concatenate(p32), np.concatenate(p16), np.concatenate(top)


def search_rd(J, S, R, cus, xy, pred, tau, qp, shortlist=True):
    """(total SSD, total bits, fraction of the lattice's work searched) of the quad-tree decisions
    at one QP: the full search when pred is None, else the pruned search of pruned_search; a CU's
    own cost counts one flag bit, a split one more"""
    lam = LAMBDA_QP(qp)
    idx = {(int(c["x"]), int(c["y"]), int(c["w"])): i for i, c in enumerate(cus)}
    work = [0.0]

    def own(x, y, s, modes):
        i = idx[(x, y, s)]
        row = J[i]
        work[0] += s * s * (len(modes) if modes is not None else N_MODES)
        m = int(np.argmin(row)) if modes is None else int(modes[int(np.argmin(row[modes]))])
        return (row[m] + lam, S[i, m], R[i, m] + 1.0)

    def add(parts):
        return (sum(p[0] for p in parts) + lam, sum(p[1] for p in parts), sum(p[2] for p in parts) + 1.0)

    def node(x, y, s, b, x0, y0):
        if pred is None:
            p, modes = 0.5, None
        else:
            p64, p32, p16, top = pred
            p = (p64[b] if s == 64 else p32[b][((y - y0) // 32) * 2 + (x - x0) // 32] if s == 32
                 else p16[b][((y - y0) // 16) * 4 + (x - x0) // 16] if s == 16 else 0.0)
            cell = ((y - y0) // 16) * 4 + (x - x0) // 16
            modes = top[b][cell] if (shortlist and s <= 16) else None
        best = None
        if not p > tau:
            best = own(x, y, s, modes)
        if s > 8 and not p < 1 - tau:
            h = s // 2
            kids = add([node(x + dx, y + dy, h, b, x0, y0) for dy in (0, h) for dx in (0, h)])
            if best is None or kids[0] < best[0]:
                best = kids
        return best

    ssd = bits = 0.0
    for b, (x0, y0) in enumerate(xy):
        r = node(int(x0), int(y0), 64, b, int(x0), int(y0))
        ssd += r[1]
        bits += r[2]
    return ssd, bits, work[0] / (len(xy) * 4 * 64 * 64 * N_MODES)


def bd_rate(rate_a, psnr_a, rate_b, psnr_b):
    """Bjontegaard delta rate (VCEG-M33) of curve b against curve a, in percent: the log rate of
    each curve as a cubic polynomial in PSNR, integrated over the PSNR interval both cover; the
    mean log-rate difference d gives (e^d - 1) * 100"""
    la, lb = np.log(np.asarray(rate_a, np.float64)), np.log(np.asarray(rate_b, np.float64))
    pa, pb = np.asarray(psnr_a, np.float64), np.asarray(psnr_b, np.float64)
    ca, cb = np.polyfit(pa, la, 3), np.polyfit(pb, lb, 3)
    lo, hi = max(pa.min(), pb.min()), min(pa.max(), pb.max())
    ia, ib = np.polyint(ca), np.polyint(cb)
    d = ((np.polyval(ib, hi) - np.polyval(ib, lo)) - (np.polyval(ia, hi) - np.polyval(ia, lo))) / (hi - lo)
    return float((np.exp(d) - 1.0) * 100.0)


def pruned_search(J, cus, xy, pred, tau, shortlist=True):
    """RD cost of the quad-tree search over the candidates the predictions keep, against the
    full search: a level is decided by the prediction only when its split probability is beyond
    tau (or below 1 - tau); 16x16 and 8x8 CUs try only their cell's shortlist.  Returns
    (relative RD-cost increase, fraction of the lattice's work (CU samples x modes) searched)."""
    p64, p32, p16, top = pred
    idx = {(int(c["x"]), int(c["y"]), int(c["w"])): i for i, c in enumerate(cus)}
    split_bits = LAMBDA_QP(32) * 1.0
    work = [0.0]

    def own(x, y, s, modes):
        row = J[idx[(x, y, s)]]
        work[0] += s * s * (len(modes) if modes is not None else N_MODES)
        return (row.min() if modes is None else row[modes].min()) + split_bits

    def full(x, y, s):
        o = J[idx[(x, y, s)]].min() + split_bits
        if s == 8:
            return o
        h = s // 2
        return min(o, sum(full(x + dx, y + dy, h) for dy in (0, h) for dx in (0, h)) + split_bits)

    def node(x, y, s, b, x0, y0):
        if s == 64:
            p = p64[b]
        elif s == 32:
            p = p32[b][((y - y0) // 32) * 2 + (x - x0) // 32]
        elif s == 16:
            p = p16[b][((y - y0) // 16) * 4 + (x - x0) // 16]
        else:
            p = 0.0
        cell = ((y - y0) // 16) * 4 + (x - x0) // 16
        modes = top[b][cell] if (shortlist and s <= 16) else None
        best = np.inf
        if not p > tau:
            best = own(x, y, s, modes)
        if s > 8 and not p < 1 - tau:
            h = s // 2
            best = min(best, sum(node(x + dx, y + dy, h, b, x0, y0) for dy in (0, h) for dx in (0, h)) + split_bits)
        return best

    jp = jf = 0.0
    for b, (x0, y0) in enumerate(xy):
        jp += node(int(x0), int(y0), 64, b, int(x0), int(y0))
        jf += full(int(x0), int(y0), 64)
    all_work = len(xy) * 4 * 64 * 64 * N_MODES
    return (jp - jf) / jf, work[0] / all_work


def prior_predictions(labels, n):
    """the method without the network: constant split probabilities (training label rates) and
    the 8 most frequent training modes as every cell's shortlist"""
    p64 = np.full(n, labels[:, 0].mean())
    p32 = np.full((n, 4), labels[:, 1:5].mean())
    p16 = np.full((n, 16), labels[:, 5:21].mean())
    freq = np.bincount(labels[:, 21:37].ravel(), minlength=N_MODES)
    top = np.tile(np.argsort(-freq)[:SHORTLIST], (n, 16, 1))
    return p64, p32, p16, top


def kept_cus(cus, xy, pred, tau):
    """the square CUs the pruned search evaluates (any of their modes)"""
    p64, p32, p16, _ = pred
    keep = []
    idx = {(int(c["x"]), int(c["y"]), int(c["w"])): i for i, c in enumerate(cus)}

    def node(x, y, s, b, x0, y0):
        p = (p64[b] if s == 64 else p32[b][((y - y0) // 32) * 2 + (x - x0) // 32] if s == 32
             else p16[b][((y - y0) // 16) * 4 + (x - x0) // 16] if s == 16 else 0.0)
        if not p > tau:
            keep.append(idx[(x, y, s)])
        if s > 8 and not p < 1 - tau:
            h = s // 2
            for dy in (0, h):
                for dx in (0, h):
                    node(x + dx, y + dy, h, b, x0, y0)

    for b, (x0, y0) in enumerate(xy):
        node(int(x0), int(y0), 64, b, int(x0), int(y0))
    return cus[np.array(sorted(keep), dtype=np.int64)]


def lattice_ms(frame, cus, qp=32, reps=3, modes=None):
    """GPU time of the intra lattice over a CU list (one QP; all 33 modes, or the per-CU mode
    lists [n][K] when given), CUDA events"""
    import torch
    from . import LAT_Q, lib
    H, W = frame.shape
    L = lib()
    L.uavs3e_cuda_intra_lattice_modes_device.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int,
                                                          C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int,
                                                          C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                                          C.c_void_p]
    if len(cus) == 0:
        return 0.0
    d = torch.from_numpy(np.ascontiguousarray(frame)).cuda()
    d_cus = torch.from_numpy(np.ascontiguousarray(cus).view(np.uint8)).cuda()
    n = len(cus)
    d_modes = None if modes is None else torch.from_numpy(np.ascontiguousarray(modes, dtype=np.uint8)).cuda()
    K = 33 if modes is None else modes.shape[1]
    d_satd = torch.empty(n * 33, dtype=torch.int32, device="cuda")
    d_q = torch.empty(n * 33 * LAT_Q.itemsize, dtype=torch.uint8, device="cuda")
    qps = np.array([qp], np.int32)
    st = torch.cuda.current_stream()

    def run():
        check(L.uavs3e_cuda_intra_lattice_modes_device(d.data_ptr(), W, d.data_ptr(), W, W, H, d_cus.data_ptr(), n,
                                                       None if d_modes is None else d_modes.data_ptr(), K, 0,
                                                       qps.ctypes.data, 1, 1, d_satd.data_ptr(), d_q.data_ptr(),
                                                       st.cuda_stream), "intra_lattice")

    run()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(st)
    for _ in range(reps):
        run()
    e1.record(st)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def pruned_lattice_ms(frame, cus, xy, pred, tau, qp=32):
    """GPU time of the pruned search's lattice work: the kept 64x64 / 32x32 CUs with all modes,
    the kept 16x16 / 8x8 CUs with their cell's shortlist"""
    kept = kept_cus(cus, xy, pred, tau)
    big = kept[kept["w"] >= 32]
    small = kept[kept["w"] <= 16]
    top = pred[3]
    origin = {(int(x), int(y)): b for b, (x, y) in enumerate(xy)}
    modes = np.zeros((len(small), SHORTLIST), np.uint8)
    for i, c in enumerate(small):
        x, y = int(c["x"]), int(c["y"])
        b = origin[(x & ~63, y & ~63)]
        modes[i] = top[b][((y & 63) // 16) * 4 + (x & 63) // 16]
    return lattice_ms(frame, big, qp) + lattice_ms(frame, small, qp, modes=modes), len(kept)


def experiment(train_seeds=range(100, 116), test_seeds=(900,), qp=32, steps=3000, batch=128, taus=(0.8, 0.9),
               seed=0, width=1920, height=1080, qps=(27, 32, 37, 42)):
    """train on the plain path's decisions over synthetic 1080p I-frames at every QP of qps,
    evaluate on held-out frames against the method without the network: at QP qp (accuracy,
    RD-cost increase, work), and over qps as a Bjontegaard delta rate of the pruned search
    against the full one; one dict of results"""
    import time
    import torch
    from .synth import intra_frame
    t0 = time.perf_counter()
    tr = [frame_dataset_qps(intra_frame(width, height, seed=s), qps) for s in train_seeds]
    te_frames = [intra_frame(width, height, seed=s) for s in test_seeds]
    te_all = [frame_dataset_qps(f, qps) for f in te_frames]
    te = [d[qp] for d in te_all]
    t_label = time.perf_counter() - t0
    ctus = np.concatenate([d[q][0] for d in tr for q in qps])
    labels = np.concatenate([d[q][1] for d in tr for q in qps])
    qarr = np.concatenate([np.full(len(d[q][0]), q, np.int32) for d in tr for q in qps])
    labels_at = {q: np.concatenate([d[q][1] for d in tr]) for q in qps}
    net = PruneNet(batch, seed=seed)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    hist = train(net, ctus, labels, qp=qarr, steps=steps, seed=seed)
    e1.record()
    torch.cuda.synchronize()
    train_ms = e0.elapsed_time(e1) / steps
    lq = labels_at[qp]
    out = {"train_ctus": int(len(ctus)), "train_qps": list(qps), "test_ctus": int(sum(len(d[0]) for d in te)),
           "steps": steps, "batch": batch,
           "label_rates": {"split64": float(lq[:, 0].mean()), "split32": float(lq[:, 1:5].mean()),
                           "split16": float(lq[:, 5:21].mean()),
                           "mode_top8_share": float(np.sort(np.bincount(lq[:, 21:37].ravel(), minlength=N_MODES))[::-1][:SHORTLIST].sum() / lq[:, 21:37].size)},
           "train_ms_per_step": train_ms, "label_s": t_label, "loss_first": hist[0], "loss_last": float(np.mean(hist[-20:]))}
    # accuracy against the held-out plain decisions at QP qp
    te_ctus = np.concatenate([d[0] for d in te])
    te_labels = np.concatenate([d[1] for d in te])
    pred = predict(net, te_ctus, qp)
    prior = prior_predictions(lq, len(te_ctus))
    for name, p in (("net", pred), ("prior", prior)):
        p64, p32, p16, top = p
        out[name] = {
            "split64_acc": float(((p64 > 0.5) == te_labels[:, 0].astype(bool)).mean()),
            "split32_acc": float(((p32 > 0.5) == te_labels[:, 1:5].astype(bool)).mean()),
            "split16_acc": float(((p16 > 0.5) == te_labels[:, 5:21].astype(bool)).mean()),
            "mode_top8_recall": float((top == te_labels[:, 21:37, None]).any(2).mean()),
        }
    # pruned search on the held-out frames at QP qp: RD-cost increase and work kept, per threshold
    for tau in taus:
        for name, p in (("net", pred), ("prior", prior)):
            dj, wk, off = [], [], 0
            for d in te:
                n = len(d[0])
                sub = tuple(a[off:off + n] for a in p)
                r = pruned_search(d[3], d[6], d[2], sub, tau)
                dj.append(r[0]); wk.append(r[1])
                off += n
            out[name][f"tau{tau}"] = {"rd_cost_increase": float(np.mean(dj)), "work_fraction": float(np.mean(wk))}
    # over the QPs: rate (bits of the RD model) and PSNR-Y (SSD of the decisions) of the full and
    # the pruned searches on the held-out frames, and the Bjontegaard delta rates
    n_pix = float(sum(len(d[0]) for d in te)) * 64 * 64
    curves = {"full": {"rate": [], "psnr": [], "work": []}}
    for tau in taus:
        curves[f"net_tau{tau}"] = {"rate": [], "psnr": [], "work": []}
        curves[f"prior_tau{tau}"] = {"rate": [], "psnr": [], "work": []}
    for q in qps:
        preds = {"net": predict(net, np.concatenate([d[q][0] for d in te_all]), q),
                 "prior": prior_predictions(labels_at[q], sum(len(d[q][0]) for d in te_all))}
        runs = [("full", None, 0.9)] + [(f"{m}_tau{tau}", m, tau) for tau in taus for m in ("net", "prior")]
        for key, m, tau in runs:
            ssd = bits = work = 0.0
            off = 0
            for d in te_all:
                c, _, xy, J, S, R, cus = d[q]
                n = len(c)
                p = None if m is None else tuple(a[off:off + n] for a in preds[m])
                off += n
                r = search_rd(J, S, R, cus, xy, p, tau, q)
                ssd += r[0]; bits += r[1]; work += r[2] / len(te_all)
            curves[key]["rate"].append(bits)
            curves[key]["psnr"].append(10.0 * np.log10(255.0 ** 2 * n_pix / max(ssd, 1.0)))
            curves[key]["work"].append(work)
    out["bd_rate"] = {"qps": list(qps), "model": "rate = the RD model's bits (coded levels, all-zero and split "
                                                  "flags), PSNR-Y of the CTUs' reconstruction by the chosen CUs/modes",
                      "curves": curves}
    for key in curves:
        if key != "full":
            out["bd_rate"][key] = {"bd_rate_pct": bd_rate(curves["full"]["rate"], curves["full"]["psnr"],
                                                          curves[key]["rate"], curves[key]["psnr"]),
                                   "mean_work_fraction": float(np.mean(curves[key]["work"]))}
    # GPU time: inference of a frame's CTUs, and the lattice over all square CUs vs the kept ones
    f0, d0 = te_frames[0], te[0]
    infer = PruneNet(len(d0[0]), params=net.params())
    x = torch.from_numpy(host_input(d0[0], qp)).to(torch.bfloat16).cuda()
    infer.acts[0].copy_(x)
    infer.forward()
    e0.record()
    for _ in range(5):
        infer.forward()
    e1.record()
    torch.cuda.synchronize()
    out["inference_ms_per_frame"] = e0.elapsed_time(e1) / 5
    full_ms = lattice_ms(f0, d0[6], qp)
    n0 = len(d0[0])
    out["lattice_square_cus_ms"] = full_ms
    out["square_cus"] = int(len(d0[6]))
    for tau in taus:
        ms, nk = pruned_lattice_ms(f0, d0[6], d0[2], tuple(a[:n0] for a in pred), tau, qp)
        out[f"pruned_lattice_tau{tau}"] = {"ms": ms, "kept_cus": int(nk), "speedup": full_ms / ms if ms else None}
    return out


def encoder_label_experiment(path, steps=2000, batch=128, seed=0):
    """the network trained on the reference encoder's own CU decisions (the fixture written by
    tests/golden/make_encoder_labels.py: seeded 512x256 I-frames coded at 4 QPs) and evaluated on
    its held-out frames against the method without the network; also how often the lattice's RD
    model (the labels of experiment()) agrees with the encoder's decisions on the same frames"""
    import torch
    from .synth import intra_frame
    d = np.load(path)
    seeds, qps, labels, xy = d["seeds"], d["qps"], d["labels"], d["xy"]
    W, H, n_train = int(d["width"]), int(d["height"]), int(d["n_train"])
    ctus = [np.stack([f[y:y + 64, x:x + 64] for x, y in xy]) for f in (intra_frame(W, H, seed=int(s)) for s in seeds)]
    nf, nq = len(seeds), len(qps)
    tr = [(f, qi) for f in range(n_train) for qi in range(nq)]
    X = np.concatenate([ctus[f] for f, _ in tr])
    Y = np.concatenate([labels[f, qi] for f, qi in tr])
    Q = np.concatenate([np.full(len(xy), int(qps[qi]), np.int32) for _, qi in tr])
    net = PruneNet(batch, seed=seed)
    hist = train(net, X, Y, qp=Q, steps=steps, seed=seed)
    out = {"frames": f"{nf} seeded {W}x{H} I-frames ({n_train} training, {nf - n_train} held out), QP "
                     f"{', '.join(str(int(q)) for q in qps)}: the reference encoder's final CUs",
           "train_samples": int(len(X)), "steps": steps, "loss_first": hist[0], "loss_last": float(np.mean(hist[-20:])),
           "encoder_label_rates": {"split64": float(Y[:, 0].mean()), "split32": float(Y[:, 1:5].mean()),
                                   "split16": float(Y[:, 5:21].mean())}}
    prior = None
    for name in ("net", "prior"):
        acc = {"split64_acc": [], "split32_acc": [], "split16_acc": [], "mode_top8_recall": []}
        for f in range(n_train, nf):
            for qi in range(nq):
                lab = labels[f, qi]
                if name == "net":
                    p64, p32, p16, top = predict(net, ctus[f], int(qps[qi]))
                else:
                    p64, p32, p16, top = prior_predictions(Y, len(lab))
                acc["split64_acc"].append(((p64 > 0.5) == lab[:, 0].astype(bool)).mean())
                acc["split32_acc"].append(((p32 > 0.5) == lab[:, 1:5].astype(bool)).mean())
                acc["split16_acc"].append(((p16 > 0.5) == lab[:, 5:21].astype(bool)).mean())
                acc["mode_top8_recall"].append((top == lab[:, 21:37, None]).any(2).mean())
        out[name] = {k: float(np.mean(v)) for k, v in acc.items()}
    # the lattice RD model's decisions on the same frames against the encoder's
    agree = {"split64": [], "split32": [], "split16": [], "mode": []}
    for f in range(nf):
        frame = intra_frame(W, H, seed=int(seeds[f]))
        dq = frame_dataset_qps(frame, tuple(int(q) for q in qps))
        for qi, q in enumerate(qps):
            pl = dq[int(q)][1]
            el = labels[f, qi]
            agree["split64"].append((pl[:, 0] == el[:, 0]).mean())
            agree["split32"].append((pl[:, 1:5] == el[:, 1:5]).mean())
            agree["split16"].append((pl[:, 5:21] == el[:, 5:21]).mean())
            agree["mode"].append((pl[:, 21:37] == el[:, 21:37]).mean())
    out["rd_model_agreement"] = {k: float(np.mean(v)) for k, v in agree.items()}
    return out


if __name__ == "__main__":
    import json
    from . import build, init
    build()
    init(0)
    print(json.dumps(experiment()))
