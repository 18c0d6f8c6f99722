"""Makes tests/golden/fmt_ref.npz: the reference's own format-word read and decode (ob_thin_read_fmt and
ob_fmt_decode, compiled from the reference's sources into oracle/_ref/libref.so by `make -C oracle ref`) on seeded
captures and soft values, for the tests on machines where the reference tree is absent.

Captures: word captures in the 64, 128 and 256 rings (spans 128, 256, 512) from lizard_gb300.synth's painter (held
to the reference's layout by tests/test_fmt_oracle.py), clean, blurred, noisy, with glare over a side, some with the
registration's mesh off by a fraction of a pixel. Each frame keeps only the pixels within 7.5 modules of the border's
outer edge (the rest set to 0), which is all the read touches, so the fixture stays small; the outputs are the
reference's on the stored frame. Soft values: a word with noise, faded sides, garbage, at each word length.

    python tests/golden/make_fmt_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))
import oracle  # noqa: E402
from lizard_gb300_testing import synth  # noqa: E402
from test_fmt_oracle import capture_cases, random_q  # noqa: E402


def border_mask(span, shape, reg):
    """Pixels whose module point (through H alone; the mesh is a fraction of a pixel) lies within 7.5 modules of the
    border's outer edge (the read's deepest samples are at 6 modules, a pixel or less to either side)."""
    h, w = shape
    Hi = np.linalg.inv(reg[:9].astype(np.float64).reshape(3, 3))
    V, U = np.mgrid[0:h, 0:w].astype(np.float64)
    q = Hi @ np.stack([U.ravel() + 0.5, V.ravel() + 0.5, np.ones(U.size)])
    mx, my = q[0] / q[2], q[1] / q[2]
    side = span + 30
    d = np.minimum(np.minimum(mx, side - mx), np.minimum(my, side - my))
    return ((d > -0.5) & (d < 7.5)).reshape(h, w)


def main():
    R = oracle.ref()
    assert R is not None, "build the reference first: make -C oracle ref"
    out = {}
    geom, words = [], []
    for c, (span, luma, reg) in enumerate(capture_cases(101, 9)):
        kept = np.where(border_mask(span, luma.shape, reg), luma, 0).astype(np.uint8)
        cells, _ = synth.fmt_geometry(span)
        q, word = np.zeros(4 * cells, np.float32), np.zeros(4, np.int32)
        R.refh_fmt_read(span, oracle._p(kept), kept.shape[1], kept.shape[0], oracle._p(reg), oracle._p(q), oracle._p(word))
        out["luma_%d" % c] = kept.ravel()
        out["reg_%d" % c] = reg
        out["q_%d" % c] = q
        geom.append((span, kept.shape[1], kept.shape[0]))
        words.append(word)
    out["count"] = np.int32(len(geom))
    out["geom"] = np.array(geom, np.int32)
    out["word"] = np.array(words, np.int32)
    rng = np.random.default_rng(202)
    dgeom, dout = [], []
    d = 0
    for span in (128, 256, 512):
        cells, nbytes = synth.fmt_geometry(span)
        for kind in ("clean", "noisy", "faded", "faded", "garbage"):
            q = random_q(rng, cells, nbytes, kind)
            vf = np.zeros(2, np.int32)
            rc = R.refh_fmt_decode(oracle._p(q), cells, nbytes, oracle._p(vf))
            out["dq_%d" % d] = q
            dgeom.append((cells, nbytes))
            dout.append((rc, *(vf if rc == 0 else (0, 0))))
            d += 1
    out["dcount"] = np.int32(d)
    out["dgeom"] = np.array(dgeom, np.int32)
    out["dout"] = np.array(dout, np.int32)
    path = os.path.join(ROOT, "tests", "golden", "fmt_ref.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes;", "words", [list(w) for w in words], "decodes", dout)


if __name__ == "__main__":
    main()
