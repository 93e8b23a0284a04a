"""Seeded parity cases shared by the golden-vector generator and the tests.

Each case is (kernel, params, seed).  Inputs are regenerated from the seed with numpy's PCG64
(identical on every platform), run through a backend object with the pyoracle method set
(pyoracle.RefLib = the reference's own C, pyoracle.Oracle = the restatement, or the GPU
table-entry adapter), and the outputs are reduced to an md5 digest.  golden.json stores the
digests the reference produced (make_golden.py).
"""
import hashlib

import numpy as np

NEIB = 576
MC_LUMA = np.array([[0, 0, 0, 64, 0, 0, 0, 0], [-1, 4, -10, 57, 19, -7, 3, -1], [-1, 4, -11, 40, 40, -11, 4, -1],
                    [-1, 3, -7, 19, 57, -10, 4, -1]], dtype=np.int8)
MC_CHROMA = np.array([[0, 64, 0, 0], [-4, 62, 6, 0], [-6, 56, 15, -1], [-5, 47, 25, -3], [-4, 36, 36, -4],
                      [-3, 25, 47, -5], [-1, 15, 56, -6], [0, 6, 62, -4]], dtype=np.int8)
SIZES = [4, 8, 16, 32, 64]


def digest(*arrays):
    h = hashlib.md5()
    for a in arrays:
        if isinstance(a, (int, np.integer)):
            a = np.array([a], dtype=np.int64)
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def pic(rng, h, w, kind):
    """test content: uniform noise, binary extremes, or smooth"""
    if kind == 0:
        return rng.integers(0, 256, (h, w), dtype=np.uint8)
    if kind == 1:
        return (rng.integers(0, 2, (h, w)) * 255).astype(np.uint8)
    y, x = np.mgrid[0:h, 0:w]
    return np.clip(128 + 60 * np.sin(x / 5.0 + rng.uniform(0, 6)) + 30 * np.cos(y / 7.0) +
                   rng.integers(-3, 4, (h, w)), 0, 255).astype(np.uint8)


# ------------------------------------------------------------------------------ runners
def run_sad(B, p, seed):
    rng = np.random.default_rng(seed)
    w, h, kind = p["w"], p["h"], p["kind"]
    o = pic(rng, h, w + 9, kind)
    r = pic(rng, h, w + 13, kind)
    return digest(B.sad(w, h, o.ctypes.data, w + 9, r.ctypes.data, w + 13),
                  B.ssd(w, h, o.ctypes.data, w + 9, r.ctypes.data, w + 13))


def run_satd_tile(B, p, seed):
    rng = np.random.default_rng(seed)
    tw, th = p["tw"], p["th"]
    out = []
    for k in range(8):
        o = pic(rng, 16, 24, k % 3)
        r = pic(rng, 16, 24, (k + 1) % 3)
        out.append(B.satd_tile(tw, th, o.ctypes.data, 24, r.ctypes.data, 24))
    return digest(np.array(out, np.int64))


def run_had(B, p, seed):
    rng = np.random.default_rng(seed)
    w, h = p["w"], p["h"]
    o = pic(rng, 64, 72, p["kind"])
    r = pic(rng, 64, 72, (p["kind"] + 1) % 3)
    return digest(B.had(w, h, o.ctypes.data, 72, r.ctypes.data, 72), B.satd_intra(w, h, o.ctypes.data, r.ctypes.data, 72, 72))


def run_ipflt(B, p, seed):
    rng = np.random.default_rng(seed)
    t, w, h = p["t"], p["w"], p["h"]
    src = pic(rng, h + 16, w + 24, p["kind"])
    s0 = src.ctypes.data + 8 * (w + 24) + 8
    taps = MC_LUMA if t in (0, 2) else MC_CHROMA
    c = taps[p["phase"]].copy()
    d = np.zeros((h, w + 5), np.uint8)
    B.ipflt(t, s0, w + 24, d.ctypes.data, w + 5, w, h, c)
    return digest(d)


def run_ipflt_ext(B, p, seed):
    rng = np.random.default_rng(seed)
    t, w, h = p["t"], p["w"], p["h"]
    src = pic(rng, h + 16, w + 24, p["kind"])
    s0 = src.ctypes.data + 8 * (w + 24) + 8
    taps = MC_LUMA if t == 0 else MC_CHROMA
    cx, cy = taps[p["px"]].copy(), taps[p["py"]].copy()
    d = np.zeros((h, w), np.uint8)
    B.ipflt_ext(t, s0, w + 24, d.ctypes.data, w, w, h, cx, cy)
    return digest(d)


def run_ipcpy(B, p, seed):
    rng = np.random.default_rng(seed)
    w, h = p["w"], p["h"]
    src = pic(rng, h, w + 7, 0)
    d = np.zeros((h, w + 3), np.uint8)
    B.ipcpy(src.ctypes.data, w + 7, d.ctypes.data, w + 3, w, h)
    return digest(d)


def padded_plane(img, pad, stride):
    h, w = img.shape
    buf = np.zeros((h + 2 * pad, stride), np.uint8)
    buf[pad:pad + h, pad:pad + w] = img
    buf[pad:pad + h, :pad] = img[:, :1]
    buf[pad:pad + h, pad + w:pad + w + pad] = img[:, -1:]
    buf[:pad] = buf[pad]
    buf[pad + h:] = buf[pad + h - 1]
    return buf


def run_if_luma_frame(B, p, seed):
    rng = np.random.default_rng(seed)
    w, h, pad = p["w"], p["h"], p["pad"]
    stride = w + 2 * pad
    p0 = padded_plane(pic(rng, h, w, p["kind"]), pad, stride).reshape(-1)
    planes = [np.zeros_like(p0) for _ in range(15)]
    base = pad * stride + pad
    B.if_luma_frame(p0.ctypes.data + base, [q.ctypes.data + base for q in planes], w, h, pad, stride)
    return digest(*planes)


def run_pel(B, p, seed):
    rng = np.random.default_rng(seed)
    w, h = p["w"], p["h"]
    o = pic(rng, h, w + 5, 0)
    r = pic(rng, h, w + 3, 0)
    res = np.zeros((h, w + 2), np.int16)
    B.pel_diff(w, h, o.ctypes.data, w + 5, r.ctypes.data, w + 3, res.ctypes.data, w + 2)
    s1 = pic(rng, h, w, 0)
    s2 = pic(rng, h, w, 1)
    av = np.zeros((h, w + 4), np.uint8)
    B.pel_avrg(w, h, av.ctypes.data, w + 4, s1.ctypes.data, s2.ctypes.data)
    resi = rng.integers(-300, 300, (h, w)).astype(np.int16)
    rec = np.zeros((2, h, w + 6), np.uint8)
    for cbf in (0, 1):
        B.recon(resi.ctypes.data, r.ctypes.data, w + 3, w, h, rec[cbf].ctypes.data, w + 6, cbf)
    return digest(res, av, rec)


def nb_array(rng, kind):
    if kind == 0:
        return rng.integers(0, 256, NEIB, dtype=np.uint8)
    if kind == 1:
        return (rng.integers(0, 2, NEIB) * 255).astype(np.uint8)
    return np.clip(128 + 50 * np.sin(np.arange(NEIB) / 9.0) + rng.integers(-4, 5, NEIB), 0, 255).astype(np.uint8)


def run_intra(B, p, seed):
    rng = np.random.default_rng(seed)
    w, h = p["w"], p["h"]
    outs = []
    for ipm in range(33):
        for avail in (0, 1, 2, 3, 7):
            for ipf in (0, 1):
                nb = nb_array(rng, (ipm + avail) % 3)
                d = np.zeros(w * h, np.uint8)
                B.intra_pred(nb, d, ipm, w, h, avail, ipf)
                outs.append(d)
    return digest(*outs)


def run_ang_entry(B, p, seed):
    rng = np.random.default_rng(seed)
    w, h = p["w"], p["h"]
    outs = []
    for mode in [m for m in range(3, 33) if m != 24]:
        nb = nb_array(rng, mode % 3)
        d = np.zeros((h, w + 6), np.uint8)
        B.ipred_ang(nb, d, w + 6, mode, w, h)
        outs.append(d)
    return digest(*outs)


def run_nbr(B, p, seed):
    rng = np.random.default_rng(seed)
    W, H = 128, 96
    img = pic(rng, H, W, p["kind"])
    i_scu = W // 4 + 2
    n_scu = i_scu * (H // 4 + 2)
    outs = []
    for t in range(40):
        w, h = int(rng.choice(SIZES)), int(rng.choice(SIZES))
        x = int(rng.integers(0, (W - w) // 4 + 1)) * 4
        y = int(rng.integers(0, (H - h) // 4 + 1)) * 4
        coded = (rng.random(n_scu) < 0.75).astype(np.uint8).reshape(H // 4 + 2, i_scu)
        coded[0, :] = coded[-1, :] = 0
        coded[:, 0] = coded[:, -1] = 0
        coded = coded.ravel().copy()
        avail = int(rng.integers(0, 8))
        if y == 0:
            avail &= ~(1 | 4)
        if x == 0:
            avail &= ~(2 | 4)
        scup = (y // 4 + 1) * i_scu + x // 4 + 1
        nb = np.zeros(NEIB, np.uint8)
        src = img.ctypes.data + y * W + x
        B.intra_get_nbr(x, y, w, h, src, W, src - W, p["lcu"], avail, nb, scup, coded, n_scu, i_scu)
        outs.append(nb)
    return digest(*outs)


def run_fdct2(B, p, seed):
    rng = np.random.default_rng(seed)
    lw, lh = p["lw"], p["lh"]
    n = (1 << lw) * (1 << lh)
    resi = rng.integers(-255, 256, n).astype(np.int16) if p["kind"] == 0 else \
        rng.integers(-32768, 32768, n).astype(np.int16)
    c = np.full(4096, 7, np.int16)
    B.trans_dct2(lw, lh, resi, c)
    coef = rng.integers(-2000, 2000, 4096).astype(np.int16) if p["kind"] == 0 else \
        rng.integers(-32768, 32768, 4096).astype(np.int16)
    r = np.zeros(4096, np.int16)
    B.itrans_dct2(lh, lw, coef, r)
    return digest(c, r)


def run_dct87(B, p, seed):
    rng = np.random.default_rng(seed)
    t, ln = p["t"], p["ln"]
    src = rng.integers(-255, 256, (1 << ln) * 8).astype(np.int16)
    outs = []
    for sh in (0, 1, 5, 8):
        d = np.zeros(4096, np.int16)
        B.trans_dct8_dst7(t, ln, src, d, sh, 8)
        outs.append(d)
    coef = rng.integers(-3000, 3000, (1 << ln) * 8).astype(np.int16)
    d = np.zeros(4096, np.int16)
    B.itrans_dct8_dst7(t, ln, coef, d, 5, 8, 32767, -32768)
    outs.append(d)
    d = np.zeros(4096, np.int16)
    B.itrans_dct8_dst7(t, ln, coef, d, 12, 8, 255, -256)
    outs.append(d)
    return digest(*outs)


def run_xform(B, p, seed):
    rng = np.random.default_rng(seed)
    lw, lh = p["lw"], p["lh"]
    n = (1 << lw) * (1 << lh)
    outs = []
    for nxn in (0, 1):
        for blk in range(4):
            for sec in range(4):
                for alt in (0, 1):
                    resi = rng.integers(-255, 256, n).astype(np.int16)
                    c = np.zeros(4096, np.int16)
                    B.transform(nxn, blk, c, resi, lw, lh, 8, sec, alt)
                    coef = (rng.integers(-60, 60, n) * (rng.random(n) < 0.3)).astype(np.int16)
                    qp = int(rng.integers(0, 64))
                    r = np.zeros(4096, np.int16)
                    B.invqt(nxn, blk, coef, r, None, None, lw, lh, qp, 8, sec, alt)
                    wq4 = rng.integers(16, 128, 16).astype(np.uint8)
                    wq8 = rng.integers(16, 128, 64).astype(np.uint8)
                    r2 = np.zeros(4096, np.int16)
                    B.invqt(nxn, blk, coef, r2, wq4, wq8, lw, lh, qp, 8, sec, alt)
                    outs += [c, r, r2]
    return digest(*outs)


def run_quant(B, p, seed):
    rng = np.random.default_rng(seed)
    outs = []
    for t in range(40):
        n = int(rng.choice([16, 64, 256, 1024, 4096]))
        coef = (rng.integers(-3000, 3000, n) * (rng.random(n) < 0.5)).astype(np.int16)
        thr = int(rng.integers(0, 100))
        outs.append(np.array([B.quant_check(coef, n, thr)], np.int64))
        qv = int(rng.integers(18, 16302))
        qb = int(rng.integers(14, 22))
        es = int(rng.integers(1, 100000))
        a = np.zeros(n, np.uint32)
        lv = np.zeros(n, np.int16)
        e = np.zeros(n, np.int64)
        last = B.quant_rdoq(coef, n, qv, qb, es, 20, a, lv, e)
        outs += [np.array([last], np.int64), a, lv, e]
    return digest(*outs)


def run_dquant(B, p, seed):
    rng = np.random.default_rng(seed)
    lw, lh = p["lw"], p["lh"]
    w, h = 1 << lw, 1 << lh
    outs = []
    for k in range(6):
        coef = (rng.integers(-400, 400, w * h) * (rng.random(w * h) < 0.4)).astype(np.int16)
        if k == 5:
            coef[:4] = [32767, -32768, 20000, -20000]
        scale = int(rng.choice([32768, 36061, 46341, 60424, 65535]))
        shift = int(rng.integers(0, 14))
        wq4 = rng.integers(16, 128, 16).astype(np.uint8)
        wq8 = rng.integers(16, 128, 64).astype(np.uint8)
        for flat in (1, 0):
            out = np.full(w * h, 99, np.int16)
            B.dquant(flat, coef, out, wq4, wq8, lw, lh, scale, shift)
            outs.append(out)
    return digest(*outs)


def run_tables(B, p, seed):
    outs = [B.dct_table(ln) for ln in range(1, 7)]
    outs += [B.scan(lw, lh) for lw in range(1, 7) for lh in range(1, 7)]
    return digest(*outs)


# ------------------------------------------------------------------ lookahead estimation
def loka_frames(rng, W, H, pocs, vel, n_rect=6):
    """4:2:0 frames of a panning scene: the frame at POC t is the W x H window of a larger
    canvas (smooth pattern + textured squares) at offset t * vel, plus per-frame noise in
    [-3, 3]; chroma = 2x-downsampled luma offset by +16 / -16 (clipped)"""
    margin = int(max(abs(vel[0]), abs(vel[1])) * max(abs(t) for t in pocs)) + 8
    CH, CW = H + 2 * margin, W + 2 * margin
    yy, xx = np.mgrid[0:CH, 0:CW]
    canvas = 128 + 45 * np.sin(xx / 9.0 + rng.uniform(0, 6)) * np.cos(yy / 13.0) + 20 * np.sin((xx + yy) / 5.0)
    for _ in range(n_rect):
        s = int(rng.integers(8, 40))
        y0, x0 = int(rng.integers(0, CH - s)), int(rng.integers(0, CW - s))
        canvas[y0:y0 + s, x0:x0 + s] = rng.integers(0, 256, (s, s))
    frames = {}
    for t in pocs:
        ox, oy = margin + int(round(t * vel[0])), margin + int(round(t * vel[1]))
        y = np.clip(canvas[oy:oy + H, ox:ox + W] + rng.integers(-3, 4, (H, W)), 0, 255).astype(np.uint8)
        c = y.reshape(H // 2, 2, W // 2, 2).astype(np.int32).mean((1, 3)).astype(np.int32)
        frames[t] = (y, np.clip(c + 16, 0, 255).astype(np.uint8), np.clip(c - 16, 0, 255).astype(np.uint8))
    return frames


LOKA_PAD = 144


def loka_inputs(p, seed):
    """(cfg record, org planes, padded reference planes) of one lookahead case"""
    import pyoracle
    rng = np.random.default_rng(seed)
    W, H, ptr = p["w"], p["h"], p.get("ptr", 8)
    l0, l1 = p["l0"], p["l1"]
    frames = loka_frames(rng, W, H, [ptr] + l0 + l1, p["vel"])
    cfg = np.zeros(1, dtype=pyoracle.LOKA_CFG)
    cfg["width"], cfg["height"], cfg["is_padding"] = W, H, p["pad"]
    cfg["max_search_range"], cfg["gop_size"], cfg["ptr"] = p["range"], p["gop"], ptr
    cfg["num_ref"][0] = [len(l0), len(l1)]
    for li, lst in enumerate((l0, l1)):
        for r, t in enumerate(lst):
            cfg["ref_ptr"][0, li, r] = t
    stride = W + 2 * LOKA_PAD
    refs = [[padded_plane(frames[t][0], LOKA_PAD, stride) for t in lst] for lst in (l0, l1)]
    return cfg, frames[ptr], refs, stride


def loka_ref_addrs(refs, stride):
    return [[r.ctypes.data + LOKA_PAD * stride + LOKA_PAD for r in lst] for lst in refs]


def run_loka(B, p, seed):
    cfg, (y, u, v), refs, stride = loka_inputs(p, seed)
    a0, a1 = loka_ref_addrs(refs, stride)
    W = p["w"]
    cost, icost, icost_uv, dqp = B.loka_estimate(cfg, y, W, u, v, W // 2, a0, a1, stride, want_uv=p["uv"],
                                                 want_dqp=p["dqp"])
    outs = [np.array([cost, icost], dtype=np.float64)]
    if icost_uv is not None:
        outs.append(np.array(icost_uv, dtype=np.float64))
    if dqp is not None:
        outs.append(dqp)
    return digest(*outs)


# ------------------------------------------------------------------ per-call TZ motion search
TZ_PAD = 144
TZ_SIZES = [(8, 8), (16, 16), (32, 32), (64, 64), (16, 8), (8, 16), (32, 16), (16, 32), (64, 32), (32, 64),
            (8, 32), (32, 8), (16, 64), (64, 16), (4, 8), (8, 4), (4, 16), (16, 4)]


def tz_planes(B, frames, pocs, W, H):
    """slot-major 16 planes (integer + 15 quarter-sample, padded by TZ_PAD) of the pictures at
    `pocs`, interpolated by the backend's own com_if_luma_frame; returns (arrays, addresses, stride)"""
    stride = W + 2 * TZ_PAD
    base = TZ_PAD * stride + TZ_PAD
    keep = []
    for t in pocs:
        p0 = padded_plane(frames[t][0], TZ_PAD, stride).reshape(-1)
        fr = [np.zeros_like(p0) for _ in range(15)]
        B.if_luma_frame(p0.ctypes.data + base, [q.ctypes.data + base for q in fr], W, H, TZ_PAD, stride)
        keep += [p0] + fr
    return keep, [a.ctypes.data + base for a in keep], stride


def tz_requests(rng, W, H, n, dists, bi_share=0.3):
    """n me_search_tz calls with the encoder's ranges of state: any MV resolution, predictors and
    bi start MVs on that resolution's grid, both cost types, adaptive raster ranges"""
    import pyoracle
    r = np.zeros(n, dtype=pyoracle.TZ_REQ)
    for i in range(n):
        w, h = TZ_SIZES[int(rng.integers(len(TZ_SIZES)))]
        mvr = int(rng.integers(0, 5))
        unit = 1 << mvr
        q = int(rng.integers(22, 46))
        r[i]["x"] = int(rng.integers(0, (W - w) // 4 + 1)) * 4
        r[i]["y"] = int(rng.integers(0, (H - h) // 4 + 1)) * 4
        r[i]["w"], r[i]["h"] = w, h
        r[i]["ref_slot"] = int(rng.integers(0, len(dists)))
        r[i]["num_refp"] = int(rng.integers(1, 5))
        r[i]["refi"] = int(rng.integers(0, r[i]["num_refp"]))
        r[i]["mvr"] = mvr
        r[i]["bi"] = int(rng.random() < bi_share)
        r[i]["flags"] = int(rng.integers(0, 4))
        r[i]["mvp"] = (rng.integers(-200, 201, 2) // unit) * unit
        r[i]["mv"] = ((r[i]["mvp"] + rng.integers(-48, 49, 2)) // unit) * unit
        r[i]["mv_ipel"] = rng.integers(-40, 41, 2)
        r[i]["other_mv"] = rng.integers(-120, 121, 2)
        r[i]["other_slot"] = int(rng.integers(0, len(dists)))
        r[i]["mot_bits_other"] = int(rng.integers(2, 24))
        r[i]["lambda_mv"] = int(np.floor(65536.0 * np.sqrt(1.43631 * 2.0 ** ((q - 16) / 4.0))))
        r[i]["dist"] = dists[r[i]["ref_slot"]]
    return r


def tz_inputs(B, p, seed):
    rng = np.random.default_rng(seed)
    W, H = p["w"], p["h"]
    frames = loka_frames(rng, W, H, [0, 4, 8], p["vel"])
    keep, addrs, stride = tz_planes(B, frames, [4, 0], W, H)
    reqs = tz_requests(rng, W, H, p["n"], [4, 8])
    pic = (W, H, p["pad"], p["range"], p["gop"])
    return pic, frames[8][0], keep, addrs, stride, reqs


def run_tz(B, p, seed):
    pic, org, keep, addrs, stride, reqs = tz_inputs(B, p, seed)
    out = B.me_tz(pic, org, p["w"], addrs, stride, reqs)
    return digest(out.view(np.uint8))


# ------------------------------------------------------------------ CU motion compensation
MC_PAD_C = 72


def mc_requests(rng, W, H, n):
    """com_mc_cu calls: CUs 8..64, one or both lists (sometimes the same picture and MV), MVs that
    reach past the picture edges, every channel selection; returns (requests, output bytes)"""
    import pyoracle
    r = np.zeros(n, dtype=pyoracle.MC_REQ)
    off = 0
    for i in range(n):
        w, h = (8, 16, 32, 64)[int(rng.integers(4))], (8, 16, 32, 64)[int(rng.integers(4))]
        r[i]["x"] = int(rng.integers(0, (W - w) // 8 + 1)) * 8
        r[i]["y"] = int(rng.integers(0, (H - h) // 8 + 1)) * 8
        r[i]["w"], r[i]["h"] = w, h
        use = int(rng.integers(1, 4))           # bit 0 list 0, bit 1 list 1
        r[i]["slot"] = [int(rng.integers(0, 2)) if use & 1 else -1, int(rng.integers(0, 2)) if use & 2 else -1]
        r[i]["mv"] = rng.integers(-260, 261, (2, 2))
        if use == 3 and rng.random() < 0.15:    # identical motion on the same picture
            r[i]["slot"][1] = r[i]["slot"][0]
            r[i]["mv"][1] = r[i]["mv"][0]
        ch = int(rng.integers(0, 3))
        r[i]["channel"] = ch
        r[i]["out_offset"] = off
        off += (w * h if ch != 2 else 0) + (w * h // 2 if ch != 1 else 0)
    return r, off


def mc_inputs(B, p, seed):
    rng = np.random.default_rng(seed)
    W, H = p["w"], p["h"]
    frames = loka_frames(rng, W, H, [0, 4, 8], p["vel"])
    keep, addrs, stride = tz_planes(B, frames, [4, 0], W, H)
    sc = W // 2 + 2 * MC_PAD_C
    chroma = [padded_plane(frames[t][c], MC_PAD_C, sc).reshape(-1) for t in (4, 0) for c in (1, 2)]
    caddrs = [a.ctypes.data + MC_PAD_C * sc + MC_PAD_C for a in chroma]
    reqs, nbytes = mc_requests(rng, W, H, p["n"])
    return (keep, addrs, stride), (chroma, caddrs, sc), reqs, nbytes


def run_mc(B, p, seed):
    (keep, addrs, stride), (chroma, caddrs, sc), reqs, nbytes = mc_inputs(B, p, seed)
    return digest(B.mc_cu(p["w"], p["h"], addrs, stride, caddrs, sc, reqs, nbytes))


def affine_requests(rng, W, H, n):
    """com_mc_cu_affine calls: CUs 16..64, 2 or 3 control points, one or both lists, 4x4 or 8x8
    sub-blocks, control-point MVs (1/16 samples) with zooms and rotations up to about +-1/4 and
    translations reaching past the picture edges; returns (requests, output bytes)"""
    import pyoracle
    r = np.zeros(n, dtype=pyoracle.AFFINE_REQ)
    off = 0
    for i in range(n):
        w, h = (16, 32, 64)[int(rng.integers(3))], (16, 32, 64)[int(rng.integers(3))]
        r[i]["x"] = int(rng.integers(0, (W - w) // 8 + 1)) * 8
        r[i]["y"] = int(rng.integers(0, (H - h) // 8 + 1)) * 8
        r[i]["w"], r[i]["h"] = w, h
        use = int(rng.integers(1, 4))
        r[i]["slot"] = [int(rng.integers(0, 2)) if use & 1 else -1, int(rng.integers(0, 2)) if use & 2 else -1]
        r[i]["cp_num"] = int(rng.integers(2, 4))
        r[i]["sub8"] = int(rng.integers(0, 2))
        for l in range(2):
            t = rng.integers(-1200, 1201, 2)                        # translation, 1/16 samples
            a = rng.uniform(-0.25, 0.25, 4)                         # affine parameters
            r[i]["cpmv"][l][0] = t
            r[i]["cpmv"][l][1] = t + np.rint(16 * w * np.array([a[0], a[1]])).astype(int)
            r[i]["cpmv"][l][2] = t + np.rint(16 * h * np.array([a[2], a[3]])).astype(int)
        r[i]["out_offset"] = off
        off += w * h * 3 // 2
    return r, off


def run_affine(B, p, seed):
    (keep, addrs, stride), (chroma, caddrs, sc), _, _ = mc_inputs(B, dict(p, n=1), seed)
    reqs, nbytes = affine_requests(np.random.default_rng(seed + 1), p["w"], p["h"], p["n"])
    return digest(B.mc_affine(p["w"], p["h"], addrs, stride, caddrs, sc, reqs, nbytes))


# ------------------------------------------------------------------ coefficient rate
def coef_models(rng, k):
    """k context models: window state 0..3, LPS probability 4..1023, MPS bit"""
    return ((rng.integers(0, 4, k) << 11) | (rng.integers(4, 1024, k) << 1) | rng.integers(0, 2, k)).astype(np.int16)


def coef_rate_inputs(rng, n):
    """blocks of levels for lbac_enc_run_length_cc_rdo: luma 4x4..64x64 and chroma 4x4..32x32,
    sparse low-frequency levels (long runs, escapes of runs >= 16 and levels >= 9, a level alone
    at the last scan position), random coder states; returns (levels, requests)"""
    import pyoracle
    r = np.zeros(n, dtype=pyoracle.COEF_RATE_REQ)
    blocks, off = [], 0
    for i in range(n):
        ch = int(rng.random() < 0.3)
        top = 5 if ch else 6
        lw, lh = int(rng.integers(2, top + 1)), int(rng.integers(2, top + 1))
        w, h = 1 << lw, 1 << lh
        kind = rng.random()
        lev = np.zeros((h, w), np.int64)
        if kind < 0.1:                                # only the last scan position
            scan = np.frombuffer(np.ctypeslib.as_array(pyoracle.Oracle().L.orc_scan(lw, lh), (w * h,)).tobytes(),
                                 np.uint16)
            lev.flat[scan[-1]] = int(rng.integers(1, 40)) * (1 if rng.random() < 0.5 else -1)
        else:
            dens = rng.uniform(0.02, 0.5)
            yy, xx = np.mgrid[0:h, 0:w]
            p = dens * np.exp(-(xx + yy) / max(2.0, rng.uniform(1.0, 0.5 * (w + h))))
            mask = rng.random((h, w)) < p
            if not mask.any():
                mask[0, 0] = True
            mag = np.where(rng.random((h, w)) < 0.1, rng.integers(9, 600, (h, w)), rng.integers(1, 9, (h, w)))
            lev = np.where(mask, mag * np.where(rng.random((h, w)) < 0.5, 1, -1), 0)
        blocks.append(lev.astype(np.int16).ravel())
        r[i]["coef_offset"] = off
        off += w * h
        r[i]["log2w"], r[i]["log2h"], r[i]["ch_type"] = lw, lh, ch
        r[i]["num_sig"] = int(np.count_nonzero(lev))
        r[i]["range"] = int(rng.integers(256, 512))
        for f, k in (("run", 12), ("run_rdoq", 12), ("level", 12), ("last1", 6), ("last2", 12)):
            r[i][f] = coef_models(rng, k)
    return np.concatenate(blocks), r


def run_coef_rate(B, p, seed):
    levels, reqs = coef_rate_inputs(np.random.default_rng(seed), p["n"])
    return digest(B.coef_rate(levels, reqs).view(np.uint8))


# ------------------------------------------------------------------ intra mode candidates (RMD)
RMD_SHAPES = [(4, 4), (8, 8), (16, 16), (32, 32), (64, 64), (8, 4), (4, 8), (16, 8), (8, 16), (32, 16), (16, 32),
              (16, 4), (4, 16), (32, 8), (8, 32), (64, 16), (16, 64), (32, 4), (4, 32), (64, 8), (8, 64)]


def rmd_ctx(rng, k):
    """k intra_dir context models: 10-bit LPS probabilities (not 0) and an MPS bit"""
    return (rng.integers(8, 1016, k) << 1) | rng.integers(0, 2, k)


def rmd_inputs(rng, n):
    """make_ipred_list calls: block shapes of every aspect (4:1 ones take 4 candidates), fast and
    full searches, DC / planar / bilinear skipped or not, MPM pairs (equal, IPCM, unsorted), LBAC
    states, inter SATDs that cut candidates or none; returns (requests, neighbour arrays, org
    blocks, avail, ipf)"""
    import pyoracle
    r = np.zeros(n, dtype=pyoracle.RMD_REQ)
    nbs, orgs, avails, ipfs = [], [], [], []
    for i in range(n):
        w, h = RMD_SHAPES[int(rng.integers(len(RMD_SHAPES)))]
        r[i]["satd_row"] = i
        r[i]["pb_w"], r[i]["pb_h"] = w, h
        m = rng.integers(0, 34, 2)
        u = rng.random()
        if u < 0.1:
            m[1] = m[0]
        elif u < 0.7:
            m = np.sort(m)
        r[i]["mpm"] = m
        r[i]["skip_ipd"] = int(rng.random() < 0.3)
        r[i]["fast"] = int(rng.random() < 0.7)
        r[i]["range"] = int(rng.integers(256, 512))
        r[i]["ctx"] = rmd_ctx(rng, 7)
        r[i]["sqrt_lambda"] = float(rng.uniform(4.0, 60.0))
        r[i]["inter_satd"] = np.iinfo(np.uint64).max if rng.random() < 0.5 else int(rng.integers(1, 40) * w * h)
        r[i]["satd_threshold"] = float(rng.uniform(0.9, 1.6))
        nbs.append(nb_array(rng, int(rng.integers(3))))
        orgs.append(pic(rng, h, w, int(rng.integers(3))))
        avails.append(int(rng.integers(0, 8)))
        ipfs.append(int(rng.integers(0, 2)))
    return r, nbs, orgs, avails, ipfs


def rmd_satd(B, reqs, nbs, orgs, avails, ipfs):
    """the 33 SATDs per block (com_intra_pred + calc_satd_intra) by backend B"""
    satd = np.zeros((len(reqs), 33), np.uint32)
    for i in range(len(reqs)):
        w, h = int(reqs[i]["pb_w"]), int(reqs[i]["pb_h"])
        d = np.zeros(w * h, np.uint8)
        for mode in range(33):
            B.intra_pred(nbs[i], d, mode, w, h, avails[i], ipfs[i])
            satd[i, mode] = B.satd_intra(w, h, orgs[i].ctypes.data, d.ctypes.data, w, w)
    return satd


def run_rmd(B, p, seed):
    rng = np.random.default_rng(seed)
    reqs, nbs, orgs, avails, ipfs = rmd_inputs(rng, p["n"])
    if hasattr(B, "make_ipred_list"):            # the reference itself, block by block
        import pyoracle
        out = np.zeros(len(reqs), dtype=pyoracle.RMD_OUT)
        for i in range(len(reqs)):
            out[i], _ = B.make_ipred_list(nbs[i], orgs[i].ctypes.data, int(reqs[i]["pb_w"]), avails[i], ipfs[i],
                                          reqs[i])
    else:
        out = B.intra_rmd(rmd_satd(B, reqs, nbs, orgs, avails, ipfs), reqs)
    return digest(out.view(np.uint8))


# ------------------------------------------------------------------ affine motion search
def affme_paint(rng, frames, W, H, n=6):
    """flat, one-directional (stripe) and nearly one-directional patches at the same place in
    every frame: blocks over them give singular or nearly singular normal equations"""
    for _ in range(n):
        s = int(rng.integers(24, 72))
        y0, x0 = int(rng.integers(0, H - s)), int(rng.integers(0, W - s))
        kind = int(rng.integers(4))
        val = int(rng.integers(30, 220))
        xx = np.arange(s)
        speck = (rng.random((s, s)) < 0.004).astype(np.uint8)
        for t in frames:
            y = frames[t][0]
            if kind == 0:
                y[y0:y0 + s, x0:x0 + s] = val
            elif kind == 1:
                y[y0:y0 + s, x0:x0 + s] = np.clip(val + 40 * np.sin(xx / 3.0), 0, 255).astype(np.uint8)[None, :]
            elif kind == 2:
                y[y0:y0 + s, x0:x0 + s] = np.clip(val + 40 * np.sin(xx / 4.0), 0, 255).astype(np.uint8)[:, None]
            else:                       # nearly one-directional: a stripe pattern with sparse specks
                y[y0:y0 + s, x0:x0 + s] = np.clip(val + 40 * np.sin(xx / 5.0), 0, 254).astype(np.uint8)[None, :] + speck


def affme_requests(rng, W, H, n, n_slots, bi_share=0.3):
    """affine_me_gradient calls as analyze_affine_uni / _bi make them: CUs 16..64, AMVR index
    0..2 with MVPs and start CPMVs on that step's grid, uni calls that pick their start from a
    quarter-sample uni MV (some far outside the picture, so mv_clip acts), bi calls against the
    other list's prediction, a few CPMVs at the 18-bit limits"""
    import pyoracle
    r = np.zeros(n, dtype=pyoracle.AFFME_REQ)
    for i in range(n):
        w, h = (16, 32, 64)[int(rng.integers(3))], (16, 32, 64)[int(rng.integers(3))]
        mvr = int(rng.integers(0, 3))
        unit = 1 << (2, 4, 0)[mvr]
        q = int(rng.integers(22, 46))
        r[i]["x"] = int(rng.integers(0, (W - w) // 8 + 1)) * 8
        r[i]["y"] = int(rng.integers(0, (H - h) // 8 + 1)) * 8
        r[i]["w"], r[i]["h"] = w, h
        r[i]["ref_slot"] = int(rng.integers(0, n_slots))
        r[i]["num_refp"] = int(rng.integers(1, 5))
        r[i]["refi"] = int(rng.integers(0, r[i]["num_refp"]))
        r[i]["mvr"] = mvr
        bi = rng.random() < bi_share
        r[i]["flags"] = (pyoracle.AFFME_BI if bi else (pyoracle.AFFME_UNI_START if rng.random() < 0.6 else 0)) | \
            (pyoracle.AFFME_SUB8 if rng.random() < 0.3 else 0)
        r[i]["other_slot"] = int(rng.integers(0, n_slots))
        r[i]["lambda_mv"] = int(np.floor(65536.0 * np.sqrt(1.43631 * 2.0 ** ((q - 16) / 4.0))))
        r[i]["mot_bits_other"] = int(rng.integers(2, 24))
        t = rng.integers(-700, 701, 2)
        if rng.random() < 0.05:
            t = np.array([131071 - int(rng.integers(0, 64)), -131072 + int(rng.integers(0, 64))])[rng.permutation(2)]
        a = rng.uniform(-0.06, 0.06, 2)
        mvp = np.array([t, t + np.rint(16 * w * a).astype(int)])
        r[i]["mvp"] = np.clip((mvp // unit) * unit, -131072, 131071 // unit * unit)
        start = r[i]["mvp"] + (rng.integers(-64, 65, (2, 2)) // unit) * unit
        r[i]["mv"] = np.clip(start, -131072, 131071 // unit * unit)
        if r[i]["flags"] & pyoracle.AFFME_UNI_START:
            um = rng.integers(-300, 301, 2) if rng.random() < 0.85 else rng.integers(-2500, 2501, 2)
            r[i]["mv"] = 0
            r[i]["mv"][0] = um
        ot = rng.integers(-500, 501, 2)
        r[i]["other_mv"] = [ot, ot + rng.integers(-40, 41, 2)]
    return r


def affme_inputs(B, p, seed):
    rng = np.random.default_rng(seed)
    W, H = p["w"], p["h"]
    frames = loka_frames(rng, W, H, [0, 4, 8], p["vel"])
    if p.get("paint"):
        affme_paint(rng, frames, W, H)
    keep, addrs, stride = tz_planes(B, frames, [4, 0], W, H)
    reqs = affme_requests(rng, W, H, p["n"], 2)
    return frames[8][0], keep, addrs, stride, reqs


def run_affme(B, p, seed):
    org, keep, addrs, stride, reqs = affme_inputs(B, p, seed)
    out = B.me_affine(p["w"], p["h"], org, p["w"], addrs, stride, reqs)
    return digest(out.view(np.uint8))


# ------------------------------------------------------------------ RDOQ of transform blocks
RDOQ_SIZES = [(2, 2), (3, 3), (4, 4), (5, 5), (6, 6), (2, 3), (3, 2), (2, 4), (4, 2), (3, 4), (4, 3), (3, 5), (5, 3),
              (4, 5), (5, 4), (4, 6), (6, 4), (5, 6), (6, 5), (3, 6), (6, 3)]


def rdoq_ests(rng, k):
    """k sets of bin-cost estimates: pairs of costs (1/32768 bit units) between ~0.01 and ~6 bits"""
    import pyoracle
    e = np.zeros(k, dtype=pyoracle.RDOQ_EST)
    for f in ("ctp", "cbf", "run", "lvl", "lst"):
        e[f] = rng.integers(300, 200000, e[f].shape)
    return e


def rdoq_inputs(B, p, seed):
    """forward DCT2 coefficients of Laplacian residual blocks of every TB shape, quantisation
    steps 10..60, intra / inter, luma / chroma"""
    import pyoracle
    rng = np.random.default_rng(seed)
    n = p["n"]
    reqs = np.zeros(n, dtype=pyoracle.RDOQ_REQ)
    parts, off = [], 0
    for i in range(n):
        lw, lh = RDOQ_SIZES[int(rng.integers(len(RDOQ_SIZES)))]
        w, h = 1 << lw, 1 << lh
        scale = float(rng.choice([2.0, 6.0, 20.0, 60.0]))
        resi = np.clip(np.rint(rng.laplace(0, scale, (h, w))), -255, 255).astype(np.int16)
        coef = np.zeros(w * h, np.int16)
        B.trans_dct2(lw, lh, resi, coef)
        parts.append(coef)
        qp = int(rng.integers(10, 61))
        reqs[i]["coef_offset"] = off
        reqs[i]["log2w"], reqs[i]["log2h"], reqs[i]["qp"] = lw, lh, qp
        reqs[i]["is_intra"] = int(rng.integers(0, 2))
        reqs[i]["ch_type"] = 0 if (lw > 5 or lh > 5) else int(rng.integers(0, 3))
        reqs[i]["slice_type"] = int(rng.integers(1, 4))
        reqs[i]["est"] = int(rng.integers(0, p["k"]))
        reqs[i]["lambda_"] = int(round(1.43631 * 2.0 ** ((qp - 16) / 4.0) * 32768))
        off += w * h
    return reqs, rdoq_ests(rng, p["k"]), np.concatenate(parts)


def wq_matrices(rng):
    """weighting matrices: 4x4 and 8x8, weights 8..255 (64 = flat)"""
    return rng.integers(8, 256, 16).astype(np.uint8), rng.integers(8, 256, 64).astype(np.uint8)


def run_quant_wq(B, p, seed):
    reqs, _, coefs = rdoq_inputs(B, dict(p, k=1), seed)
    wq4, wq8 = wq_matrices(np.random.default_rng(seed + 1))
    nz = B.quant_wq(reqs, wq4, wq8, coefs)
    return digest(nz, coefs)


def affmvp_inputs(p, seed):
    """a motion field in the reference's layout (stride w + 2, one border row / column of invalid
    reference indices), reference POCs on both sides of the current picture and CU requests of
    every width, list, reference index and AMVR index"""
    import pyoracle
    rng = np.random.default_rng(seed)
    w, h, nref = p["w"], p["h"], p["nref"]
    i_scu, rows = w + 2, h + 2
    refi = np.full((rows, i_scu, 2), -1, dtype=np.int8)
    inner = rng.integers(0, nref, (h, w, 2))
    inner[rng.random((h, w, 2)) < 0.35] = -1
    refi[1:h + 1, 1:w + 1] = inner
    mv = rng.integers(-300, 301, (rows, i_scu, 2, 2))
    if p.get("big"):
        wide = rng.random((rows, i_scu, 2, 2)) < 0.3
        mv[wide] = rng.integers(-32768, 32768, int(wide.sum()))
    ptr_cur = 40
    ref_ptr = np.zeros((nref, 2), dtype=np.int64)
    for i in range(nref):
        ref_ptr[i, 0] = ptr_cur - (1 << i) if i % 2 == 0 else ptr_cur - 3 * i
        ref_ptr[i, 1] = ptr_cur + (1 << i) if i % 3 else ptr_cur - 5 - i
    n = p["n"]
    reqs = np.zeros(n, dtype=pyoracle.AFFMVP_REQ)
    widths = [c for c in (8, 16, 32, 64, 128) if c // 4 <= w]
    for k in range(n):
        cw = int(rng.choice(widths))
        x = int(rng.integers(0, w - cw // 4 + 1))
        y = int(rng.integers(0, h))
        reqs[k] = (y * i_scu + x, cw, int(rng.integers(0, 2)), int(rng.integers(0, nref)), int(rng.integers(0, 3)),
                   (0, 0, 0))
    return ptr_cur, ref_ptr, mv.astype(np.int16).reshape(-1, 2, 2), refi.reshape(-1, 2), i_scu, reqs


def run_affmvp(B, p, seed):
    ptr_cur, ref_ptr, mv, refi, i_scu, reqs = affmvp_inputs(p, seed)
    res = B.affine_mvp(ptr_cur, ref_ptr, mv, refi, i_scu, reqs)
    out = res[0] if isinstance(res, tuple) else res
    return digest(out)


def affmrg_inputs(p, seed):
    """a picture's coded-CU maps in the reference's layout (stride w + 2, border of uncoded SCUs):
    64x64 CTUs split into random CUs (8..64), each inter (some affine: 4- or 6-parameter, 16x16
    and larger) or intra, with per-list reference indices and per-SCU MVs; the colocated picture's
    list-0 maps; merge requests of every affine CU size at random positions"""
    import pyoracle
    rng = np.random.default_rng(seed)
    w, h = p["w"], p["h"]
    i_scu, rows = w + 2, h + 2
    org = i_scu + 1
    scu = np.zeros(rows * i_scu, np.uint8)
    pos = np.zeros(rows * i_scu, np.uint32)
    refi = np.full((rows * i_scu, 2), -1, np.int8)
    mv = np.zeros((rows * i_scu, 2, 2), np.int16)

    def cu(x, y, s):
        # a CU crossing the picture's edge is split, as the encoder does
        if s > 2 and (x + s > w or y + s > h or rng.random() < (0.6 if s > 4 else 0.4)):
            for dy in (0, s // 2):
                for dx in (0, s // 2):
                    cu(x + dx, y + dy, s // 2)
            return
        cw = ch = s
        if s >= 4 and rng.random() < 0.3:   # a horizontal or vertical binary split
            if rng.random() < 0.5:
                ch = s // 2
                cus = [(x, y, cw, ch), (x, y + ch, cw, ch)]
            else:
                cw = s // 2
                cus = [(x, y, cw, ch), (x + cw, y, cw, ch)]
        else:
            cus = [(x, y, cw, ch)]
        for (cx, cy, a, b) in cus:
            if cx >= w or cy >= h:
                continue
            intra = rng.random() < 0.2
            aff = 0 if intra or a < 4 or b < 4 or rng.random() < 0.55 else int(rng.integers(1, 3))
            r = np.where(rng.random(2) < 0.65, 0, rng.integers(-1, p["nref"], 2))
            if not intra and (r < 0).all():
                r[rng.integers(0, 2)] = rng.integers(0, p["nref"])
            base = rng.integers(-200, 201, (2, 2))
            lw, lh = int(a * 4).bit_length() - 1, int(b * 4).bit_length() - 1
            for yy in range(cy, min(cy + b, h)):
                for xx in range(cx, min(cx + a, w)):
                    k = org + yy * i_scu + xx
                    scu[k] = 1 | (2 if intra else 0) | (aff << 4)
                    pos[k] = ((cy * i_scu + cx) << 6) | (lh << 3) | lw
                    if not intra:
                        refi[k] = r
                        mv[k] = base + rng.integers(-24, 25, (2, 2))

    for cy in range(0, h, 16):
        for cx in range(0, w, 16):
            cu(cx, cy, 16)
    col_refi = np.full((rows * i_scu, 2), -1, np.int8)
    col_mv = np.zeros((rows * i_scu, 2, 2), np.int16)
    inner = np.zeros((rows, i_scu), bool)
    inner[1:h + 1, 1:w + 1] = True
    inner = inner.ravel()
    col_refi[inner, 0] = rng.integers(-1, 4, int(inner.sum()))
    col_mv[inner, 0] = rng.integers(-300, 301, (int(inner.sum()), 2))
    pic = np.zeros(1, dtype=pyoracle.AFFMRG_PIC)
    pic["ptr"] = 40
    b = p["slice"] == "B"
    pic["ref0_ptr"] = (32, 48) if b else (36, 28)
    pic["col_list_ptr"] = np.array([(16, 24, 8, 0)[i % 4] if b else (20, 12, 4, 34)[i % 4] for i in range(17)])
    pic["i_scu"] = i_scu
    pic["pic_width_in_scu"] = w
    pic["pic_height_in_scu"] = h
    pic["rows"] = rows
    pic["slice_type"] = 3 if b else 2
    pic["log2_max_cuwh"] = 6
    n = p["n"]
    reqs = np.zeros(n, dtype=pyoracle.AFFMRG_REQ)
    sizes = [16, 32, 64]
    for k in range(n):
        cw, ch = int(rng.choice(sizes)), int(rng.choice(sizes))
        x = int(rng.integers(0, w - cw // 4 + 1)) & ~(cw // 4 - 1)
        y = int(rng.integers(0, h - ch // 4 + 1)) & ~(ch // 4 - 1)
        reqs[k] = (y * i_scu + x, cw, ch)
    return pic, mv.reshape(-1, 2, 2), refi, scu, pos, col_mv, col_refi, reqs


def run_affmrg(B, p, seed):
    pic, mv, refi, scu, pos, cmv, crefi, reqs = affmrg_inputs(p, seed)
    res = B.affine_merge(pic, mv, refi, scu, pos, cmv, crefi, reqs)
    out = res[0] if isinstance(res, tuple) else res
    return digest(out)


def run_rdoq(B, p, seed):
    reqs, ests, coefs = rdoq_inputs(B, p, seed)
    nz = B.rdoq(reqs, ests, coefs)
    return digest(coefs, nz)


RUNNERS = {
    "sad": run_sad, "satd_tile": run_satd_tile, "had": run_had, "ipflt": run_ipflt, "ipflt_ext": run_ipflt_ext,
    "ipcpy": run_ipcpy, "if_luma_frame": run_if_luma_frame, "pel": run_pel, "intra": run_intra,
    "ang_entry": run_ang_entry, "nbr": run_nbr, "fdct2": run_fdct2, "dct87": run_dct87, "xform": run_xform,
    "quant": run_quant, "dquant": run_dquant, "tables": run_tables, "loka": run_loka, "tz": run_tz, "mc": run_mc, "affine": run_affine, "affme": run_affme, "rmd": run_rmd, "coef_rate": run_coef_rate, "quant_wq": run_quant_wq, "affmvp": run_affmvp, "affmrg": run_affmrg, "rdoq": run_rdoq,
}

# TZ search cases: encoder core search (padded references, random-access and low-delay ranges)
# and one without padding
TZ_CASES = [
    dict(w=192, h=128, pad=1, range=384, gop=16, vel=(2.5, -1.25), n=96),
    dict(w=160, h=96, pad=1, range=64, gop=4, vel=(-4.0, 3.0), n=96),
    dict(w=128, h=128, pad=0, range=384, gop=16, vel=(1.75, 2.5), n=64),
]

# CU motion-compensation cases
MC_CASES = [
    dict(w=192, h=128, vel=(2.5, -1.25), n=160),
    dict(w=96, h=64, vel=(-6.0, 3.5), n=96),
]

# affine motion search cases: panning content, and the same with flat and stripe patches
AFFME_CASES = [
    dict(w=192, h=128, vel=(2.5, -1.25), n=96),
    dict(w=160, h=96, vel=(-3.0, 2.0), n=96, paint=1),
]

# weighted quantisation cases (quant_non_zero with pic_wq_enable)
QUANT_WQ_CASES = [dict(n=200), dict(n=120)]

# affine control-point MVP cases (com_get_affine_mvp_scaling): a 4-reference field with small
# MVs, and a narrow 2-reference field with full-range MVs (the s16 and CPMV clips)
AFFMVP_CASES = [dict(w=48, h=32, nref=4, n=200), dict(w=30, h=17, nref=2, n=160, big=1)]

# affine merge candidate cases: B and P slices (colocated list-1 / list-0 picture), two picture
# sizes
AFFMRG_CASES = [
    dict(w=48, h=32, nref=3, slice="B", n=240),
    dict(w=64, h=48, nref=2, slice="P", n=240),
]

# coefficient rate cases (lbac_enc_run_length_cc_rdo)
COEF_RATE_CASES = [dict(n=200), dict(n=150)]

# intra mode candidate cases (make_ipred_list)
RMD_CASES = [dict(n=200), dict(n=120)]

# RDOQ cases (transform blocks of every shape, several estimate sets)
RDOQ_CASES = [dict(n=200, k=4), dict(n=120, k=1)]

# lookahead cases: encoder picture level (padded references, random access with both lists or
# low delay with 4 references) and the scene-cut estimate (1 reference, no padding)
LOKA_CASES = [
    dict(w=128, h=96, pad=1, range=384, gop=16, l0=[0, 4], l1=[16, 12], vel=(1.5, -0.75), uv=True, dqp=True),
    dict(w=144, h=80, pad=1, range=384, gop=16, l0=[0], l1=[16], vel=(5.0, 3.0), uv=True, dqp=True),
    dict(w=128, h=64, pad=1, range=64, gop=4, l0=[7, 6, 5, 4], l1=[], vel=(2.5, 1.25), uv=True, dqp=True),
    dict(w=136, h=72, pad=0, range=384, gop=16, l0=[7], l1=[], vel=(3.0, -2.0), uv=False, dqp=False),
    dict(w=160, h=96, pad=0, range=64, gop=4, l0=[6], l1=[], vel=(-6.0, 4.0), uv=False, dqp=False),
    dict(w=48, h=32, pad=1, range=384, gop=16, l0=[0], l1=[16], vel=(2.0, 1.0), uv=True, dqp=True),
]


def all_cases():
    cases = []
    s = 1000

    def add(kernel, **p):
        nonlocal s
        s += 1
        cases.append({"kernel": kernel, "params": p, "seed": s})

    for w in (4, 8, 16, 32, 64, 128):
        for h in (4, 8, 16, 32, 64):
            add("sad", w=w, h=h, kind=(w + h) % 3)
    for tw, th in ((4, 4), (8, 8), (16, 8), (8, 16), (8, 4), (4, 8)):
        add("satd_tile", tw=tw, th=th)
    for w in SIZES + [12, 24, 48]:
        for h in SIZES + [12, 24, 48]:
            if (w & (w - 1)) and (h & (h - 1)) and w != h:
                pass
            add("had", w=w, h=h, kind=(w * h) % 3)
    for t in range(4):
        for w in (4, 8, 16, 32, 64, 128):
            add("ipflt", t=t, w=w, h=[4, 8, 16, 32, 64][(w + t) % 5], phase=1 + (w + t) % 3, kind=t % 3)
    for t in range(2):
        for w in SIZES:
            add("ipflt_ext", t=t, w=w, h=[4, 8, 16, 32, 64][(w // 4 + t) % 5], px=1 + w % 3, py=1 + (w // 4) % 3,
                kind=w % 3)
    for w in (4, 8, 16, 32, 64, 128):
        add("ipcpy", w=w, h=8 + w % 5)
    add("if_luma_frame", w=32, h=16, pad=16, kind=0)
    add("if_luma_frame", w=40, h=24, pad=20, kind=2)
    for w in SIZES:
        add("pel", w=w, h=[4, 8, 16][w % 3])
    for w in SIZES:
        for h in SIZES:
            if (w, h) == (64, 4):
                continue   # the reference's mode-23 kernel writes past a 64x4 block (not a size it predicts)
            add("intra", w=w, h=h)
            add("ang_entry", w=w, h=h)
    for k in range(3):
        add("nbr", kind=k, lcu=64 if k < 2 else 1 << 20)
    for lw in range(2, 7):
        for lh in range(2, 7):
            if (lw, lh) in ((6, 2), (2, 6)):
                continue
            add("fdct2", lw=lw, lh=lh, kind=0)
            add("fdct2", lw=lw, lh=lh, kind=1)
    for t in (0, 1):
        for ln in range(2, 7):
            add("dct87", t=t, ln=ln)
    for lw in range(2, 6):
        for lh in range(2, 6):
            add("xform", lw=lw, lh=lh)
    add("quant")
    for lw in range(2, 7):
        for lh in range(2, 7):
            add("dquant", lw=lw, lh=lh)
    add("tables")
    for p in LOKA_CASES:
        add("loka", **p)
    for p in TZ_CASES:
        add("tz", **p)
    for p in MC_CASES:
        add("mc", **p)
    for p in MC_CASES:
        add("affine", **p)
    for p in RDOQ_CASES:
        add("rdoq", **p)
    for p in AFFME_CASES:
        add("affme", **p)
    for p in RMD_CASES:
        add("rmd", **p)
    for p in COEF_RATE_CASES:
        add("coef_rate", **p)
    for p in QUANT_WQ_CASES:
        add("quant_wq", **p)
    for p in AFFMVP_CASES:
        add("affmvp", **p)
    for p in AFFMRG_CASES:
        add("affmrg", **p)
    return cases


def run_case(B, case):
    return RUNNERS[case["kernel"]](B, case["params"], case["seed"])
