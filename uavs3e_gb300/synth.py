"""Seeded synthetic 8-bit luma sequences with the shapes and statistics of the benchmark
workloads (the external test sequences are not available; these stand in for them).

motion_sequence:  128 + 40 sin(x'/17) cos(y'/23) + U[-8, 8] noise, with (x', y') panned by a
                  global motion per frame, plus textured 48x48 rectangles (U[0, 255] texture)
                  translating at their own sub-sample velocities (rounded to whole samples).
intra_frame:      smooth gradients + stripes at 8 seeded orientations + N(0, 6^2) noise.
"""
import numpy as np


def motion_sequence(width, height, n_frames, seed=0, n_rects=12, pan=(3.25, -1.5), rect_vel=None):
    rng = np.random.default_rng(seed)
    if rect_vel is None:
        rect_vel = [(rng.uniform(-3, 3), rng.uniform(-3, 3)) for _ in range(n_rects)]
    rects = []
    for i in range(n_rects):
        tex = rng.integers(0, 256, (48, 48), dtype=np.int32)
        x0, y0 = rng.uniform(0, max(1, width - 48)), rng.uniform(0, max(1, height - 48))
        rects.append((tex, x0, y0) + tuple(rect_vel[i]))
    ys, xs = np.mgrid[0:height, 0:width].astype(np.float64)
    frames = np.empty((n_frames, height, width), dtype=np.uint8)
    for t in range(n_frames):
        base = 128 + 40 * np.sin((xs - pan[0] * t) / 17.0) * np.cos((ys - pan[1] * t) / 23.0)
        img = np.rint(base).astype(np.int32) + rng.integers(-8, 9, (height, width))
        for tex, x0, y0, vx, vy in rects:
            px, py = int(round(x0 + vx * t)), int(round(y0 + vy * t))
            xa, ya = max(px, 0), max(py, 0)
            xb, yb = min(px + 48, width), min(py + 48, height)
            if xa < xb and ya < yb:
                img[ya:yb, xa:xb] = tex[ya - py:yb - py, xa - px:xb - px]
        frames[t] = np.clip(img, 0, 255).astype(np.uint8)
    return frames


def config0_sequence(seed=0, n_frames=8):
    """416x240 luma of the CPU-runnable configuration: 2 rectangles, no pan."""
    return motion_sequence(416, 240, n_frames, seed=seed, n_rects=2, pan=(0.0, 0.0),
                           rect_vel=[(1.25, 0.5), (-0.75, 2.0)])


def intra_frame(width, height, seed=0):
    rng = np.random.default_rng(seed)
    ys, xs = np.mgrid[0:height, 0:width].astype(np.float64)
    img = 128 + 50 * (xs / width - 0.5) + 30 * np.sin(ys / height * np.pi)
    angles = rng.uniform(0, np.pi, 8)
    for k, a in enumerate(angles):
        # stripes restricted to a band of the frame so orientations vary across it
        period = rng.uniform(6, 40)
        band = (np.abs(((xs * np.cos(a) + ys * np.sin(a)) / (width + height)) * 8 - k) < 1.2)
        img += band * 35 * np.sin(2 * np.pi * (xs * np.cos(a) + ys * np.sin(a)) / period)
    img += rng.normal(0, 6, (height, width))
    return np.clip(np.rint(img), 0, 255).astype(np.uint8)


def lambda_mv_for_qp(qp):
    """The encoder's per-CTU MV lambda for an 8-bit QP: lambda = 1.43631 * 2^((qp - 16) / 4),
    lambda_mv = floor(65536 * sqrt(lambda)) (src/uavs3e.c:834, 851)."""
    lam = 1.43631 * 2.0 ** ((qp - 16.0) / 4.0)
    return int(np.floor(65536.0 * np.sqrt(lam)))
