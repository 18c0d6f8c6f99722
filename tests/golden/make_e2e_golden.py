"""Generates tests/golden/e2e_ref.npz: the reference's own whole receiver (lizard_acquire then lizard_finish, compiled
from its sources by oracle/Makefile, x86-64 build) on synthetic captures, so the GPU receiver can be held to the
reference's decode, frame by frame, on a GPU host where the reference tree is absent.

Run from the repo root where the reference is present: python tests/golden/make_e2e_golden.py

Captures (the reference's own sender paints every symbol: lizard_encode + lizard_paint_grey on seeded blocks):
  c1_*  the plain receiver's configuration: LIZARD-64 (n = 384) in the 64 ring, pasted axis-aligned and centred into
        a 1280 x 720 frame of mid-grey, AWGN sigma = 2 grey levels, seed a frame;
  c4_*  the distorted full receiver's: LIZARD-1024 (n = 1536) in the 128 ring seen by a camera in a 1920 x 1080 frame
        (rotation U(+-15 deg), tilt U(+-20 deg), the layout's side 1000 px x U(0.8, 1.1)), radial k1 about the frame
        centre, Gaussian blur in linear light (gamma 2.2), AWGN sigma = 3, seed a frame; blur 1.5 px / k1 0.03 and
        blur 0.5 px / k1 +-0.03.
For each frame: the pixels the picture's samples can read (the layout's bounding box in the frame plus a margin,
checked: the reference's own sampler reads the same grid from the crop alone), the registration the reference's
acquisition held (H, then the node mesh's (dx, dy)), and what its finish decoded: the blocks verified, each block's
LDPC iterations, the verified bytes.
"""
import lzma
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
import oracle  # noqa: E402
from lizard_gb300_testing import synth  # noqa: E402

QUIET = 2   # the painted square's quiet margin, modules a side


class _Fmt:
    def __init__(self, n, span):
        self.n, self.span = n, span


def render(grey, pxm, span, width, height, H, k1, blur, sigma, rng, mid=128, gamma=2.2):
    """The painted square (quiet margin included) seen through H (layout modules -> image pixels), radial k1, blur in
    linear light, AWGN; 8 bits."""
    from scipy.ndimage import gaussian_filter
    Wd = grey.shape[0]
    drive = grey.astype(np.float64)
    Hi = np.linalg.inv(np.asarray(H, np.float64).reshape(3, 3))
    V, U = np.mgrid[0:height, 0:width].astype(np.float64)
    ui, vi = synth._unradial(U.ravel() + 0.5, V.ravel() + 0.5, width, height, k1)
    q = Hi @ np.stack([ui, vi, np.ones(ui.size)])
    sx, sy = (q[0] / q[2] + QUIET) * pxm - 0.5, (q[1] / q[2] + QUIET) * pxm - 0.5
    inside = (sx >= 0) & (sy >= 0) & (sx <= Wd - 1.001) & (sy <= Wd - 1.001)
    x0 = np.clip(np.floor(sx).astype(np.int64), 0, Wd - 2)
    y0 = np.clip(np.floor(sy).astype(np.int64), 0, Wd - 2)
    fx, fy = np.clip(sx - x0, 0, 1), np.clip(sy - y0, 0, 1)
    val = (drive[y0, x0] * (1 - fx) + drive[y0, x0 + 1] * fx) * (1 - fy) + (drive[y0 + 1, x0] * (1 - fx) + drive[y0 + 1, x0 + 1] * fx) * fy
    img = np.where(inside, val, float(mid)).reshape(height, width)
    if blur > 0:
        img = 255.0 * np.clip(gaussian_filter((img / 255.0) ** gamma, blur, mode="nearest"), 0, 1) ** (1.0 / gamma)
    return np.clip(np.rint(img + sigma * rng.standard_normal(img.shape)), 0, 255).astype(np.uint8)


def case_c1(seed):
    r = oracle.RefFmt(384, 64, 128)
    _, grey = r.encode(oracle.spec_blocks(r.blocks, seed=seed), 0)
    W = grey.shape[0]
    frame = np.full((720, 1280), 128.0)
    oy, ox = (720 - W) // 2, (1280 - W) // 2
    frame[oy:oy + W, ox:ox + W] = grey
    rng = np.random.default_rng(seed)
    return r, 128, np.clip(np.rint(frame + 2.0 * rng.standard_normal(frame.shape)), 0, 255).astype(np.uint8)


def case_c4(seed, k1, blur):
    r = oracle.RefFmt(1536, 1024, 256)
    _, grey = r.encode(oracle.spec_blocks(r.blocks, seed=seed), 0)
    rng = np.random.default_rng(seed)
    view = synth.distorted_view(_Fmt(1536, 256), 1920, 1080, rng, base_side=1000.0)
    return r, 256, render(grey, r.pxm, 256, 1920, 1080, view, k1, blur, 3.0, rng)


def crop_box(H, nodes, span, w, h, margin=6):
    """The frame's pixels a sample of the picture can read: the layout's square through H, moved by at most the
    mesh's largest displacement, plus a margin; clamped to the frame."""
    side = span + 30
    c = np.array([[0, 0, 1], [side, 0, 1], [side, side, 1], [0, side, 1]], np.float64).T
    q = np.asarray(H, np.float64).reshape(3, 3) @ c
    u, v = q[0] / q[2], q[1] / q[2]
    d = float(np.abs(nodes).max()) if nodes.size else 0.0
    x0, x1 = int(np.floor(u.min() - d)) - margin, int(np.ceil(u.max() + d)) + margin
    y0, y1 = int(np.floor(v.min() - d)) - margin, int(np.ceil(v.max() + d)) + margin
    return max(x0, 0), max(y0, 0), min(x1, w), min(y1, h)


def main():
    oracle.build(ref=True)
    cases = [("c1_%d" % s, case_c1, (s,)) for s in range(4)]
    cases += [("c4_%d" % s, case_c4, (s, k1, b)) for s, k1, b in [(0, 0.03, 1.5), (1, 0.03, 1.5), (12, 0.03, 0.5), (21, -0.03, 0.5)]]
    out = {}
    for tag, fn, args in cases:
        r, span, luma = fn(*args)
        d = r.decode_frame(luma)
        assert d["good"] >= 0, tag + ": the reference found no symbol"
        h, w = luma.shape
        x0, y0, x1, y1 = crop_box(d["H"], d["nodes"], span, w, h)
        crop = luma[y0:y1, x0:x1].copy()
        back = np.zeros_like(luma)
        back[y0:y1, x0:x1] = crop
        g_full, s_full, _ = r.sample_decode(luma, d["H"], d["nodes"])
        g_crop, s_crop, _ = r.sample_decode(back, d["H"], d["nodes"])
        assert np.array_equal(g_full, g_crop) and np.array_equal(s_full, s_crop), tag + ": the crop misses pixels the sampler reads"
        fin = r.finish_grid(g_full)
        out[tag + "_fmt"] = np.array([r.n, r.subch, span, w, h, x0, y0, x1, y1], np.int32)
        out[tag + "_crop"] = np.frombuffer(lzma.compress(crop.tobytes(), preset=9), np.uint8)
        out[tag + "_reg"] = np.concatenate([d["H"], d["nodes"].ravel()]).astype(np.float32)
        out[tag + "_ok"] = d["ok"]
        out[tag + "_its"] = d["its"]
        out[tag + "_blocks"] = d["blocks"][d["ok"] > 0]
        print(tag, "verified", int(d["ok"].sum()), "of", r.blocks, "crop", crop.shape, "lzma", out[tag + "_crop"].size,
              "finish(grid) same set:", np.array_equal(fin["ok"], d["ok"]))
    path = os.path.join(ROOT, "tests", "golden", "e2e_ref.npz")
    np.savez(path, **out)
    print(path, os.path.getsize(path))


if __name__ == "__main__":
    main()
