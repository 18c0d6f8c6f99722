"""The format word's oracle (oracle/oracle_fmt.c) held to the reference: its Reed-Solomon code against the
reference's own rs.c, the word's soft decode against its fmt.c, the read off a capture against its
ob_thin_read_fmt (all compiled here from the reference's sources, oracle/_ref/libref.so), and the test painter
(lizard_gb300.synth's border and word) against the reference's layout. Where the reference tree is absent (the GPU
box), the committed fixture tests/golden/fmt_ref.npz holds the oracle to the reference's outputs instead."""
import ctypes
import os

import numpy as np
import pytest

import oracle
from lizard_gb300_testing import synth

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "fmt_ref.npz")
SPANS = (128, 256, 512)


def _ref():
    r = oracle.ref()
    if r is None:
        pytest.skip("the reference tree is not here")
    return r


def hard_bytes(q, cells, nbytes):
    out = np.zeros(nbytes, np.uint8)
    for k in range(nbytes):
        qs = q[(k & 3) * cells + 8 * (k >> 2):][:8]
        out[k] = sum(int(s > 0) << (7 - b) for b, s in enumerate(qs))
    return out


def test_rs_matches_reference():
    """Errors only and errors with erasures, at every word length, past the code's distance too: the same return and
    the same bytes as the reference's rs_decode / rs_decode_er."""
    R, P = _ref(), oracle.port()
    rng = np.random.default_rng(1)
    for nbytes in (16, 32, 64):
        nroots = nbytes - 3
        for trial in range(300):
            data = rng.integers(0, 256, 3, dtype=np.uint8)
            cw = np.zeros(nbytes, np.uint8)
            cw[:3] = data
            cw2 = cw.copy()
            P.orc_rs_encode(oracle._p(cw), 3, nroots)
            R.rs_encode(oracle._p(cw2), 3, nroots)
            assert np.array_equal(cw, cw2)
            nerr = int(rng.integers(0, nroots // 2 + 6))
            bad = cw.copy()
            where = rng.choice(nbytes, nerr, replace=False)
            bad[where] ^= rng.integers(1, 256, nerr, dtype=np.uint8)
            a, b = bad.copy(), bad.copy()
            ra, rb = P.orc_rs_decode(oracle._p(a), nbytes, nroots), R.rs_decode(oracle._p(b), nbytes, nroots)
            assert ra == rb and (ra < 0 or np.array_equal(a, b)), (nbytes, nerr)
            neras = int(rng.integers(0, nroots + 2))
            eras = rng.permutation(nbytes)[:min(neras, nbytes)].astype(np.int32)
            a, b = bad.copy(), bad.copy()
            ra = P.orc_rs_decode_er(oracle._p(a), nbytes, nroots, oracle._p(eras), eras.size)
            rb = R.rs_decode_er(oracle._p(b), nbytes, nroots, oracle._p(eras), eras.size)
            assert ra == rb and (ra < 0 or np.array_equal(a, b)), (nbytes, nerr, eras.size)


def random_q(rng, cells, nbytes, kind):
    """Soft values as the read leaves them, +-0.5 clipped: a word with noise, sides faded toward 0 with their bits
    flipped at random (glare), or garbage."""
    q = np.zeros(4 * cells, np.float32)
    if kind == "garbage":
        return rng.uniform(-0.5, 0.5, 4 * cells).astype(np.float32)
    span = {32: 128, 64: 256, 128: 512}[cells]
    cw = np.frombuffer(synth.fmt_word(int(rng.integers(4, 65)), int(rng.integers(0, 256)), span), np.uint8)
    for s in range(4):
        for i in range(cells):
            k = 4 * (i >> 3) + s
            bit = (cw[k] >> (7 - (i & 7))) & 1 if k < nbytes else 0
            q[s * cells + i] = 0.4 if bit else -0.4
    q += rng.normal(0, 0.15 if kind == "noisy" else 0.05, q.size).astype(np.float32)
    if kind == "faded":
        for s in rng.choice(4, int(rng.integers(1, 4)), replace=False):
            seg = q[s * cells:(s + 1) * cells]
            seg *= np.float32(rng.uniform(0.0, 0.1))
            flip = rng.random(cells) < 0.5
            seg[flip] = -seg[flip]
    return np.clip(q, -0.5, 0.5).astype(np.float32)


def test_fmt_decode_matches_reference():
    R, P = _ref(), oracle.port()
    rng = np.random.default_rng(2)
    seen = {}
    for span in SPANS:
        cells, nbytes = synth.fmt_geometry(span)
        for trial in range(120):
            kind = ("noisy", "faded", "garbage", "clean")[trial % 4]
            q = random_q(rng, cells, nbytes, kind)
            a, b = np.zeros(2, np.int32), np.zeros(2, np.int32)
            ra = P.orc_fmt_decode(oracle._p(q), cells, nbytes, oracle._p(a))
            rb = R.refh_fmt_decode(oracle._p(q), cells, nbytes, oracle._p(b))
            assert ra == rb and (ra < 0 or np.array_equal(a, b)), (span, kind, trial)
            hard = hard_bytes(q, cells, nbytes)
            h = hard.copy()
            path = "hard" if P.orc_rs_decode(oracle._p(h), nbytes, nbytes - 3) >= 0 and ra == 0 else ("erasures" if ra == 0 else "none")
            seen[path] = seen.get(path, 0) + 1
    assert seen.get("erasures", 0) > 0 and seen.get("none", 0) > 0 and seen.get("hard", 0) > 0, seen


def test_painter_matches_reference():
    """The test painter's border (corner marks, line, track, word cells) and word: the reference's layout cell for
    cell, its codeword byte for byte."""
    R = _ref()
    R.ref_fmt_new.restype = ctypes.c_void_p
    R.ref_fmt_new.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int]
    R.refh_layout_kind.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    R.ref_fmt_free.argtypes = [ctypes.c_void_p]
    for span, n, subch in ((128, 384, 64), (256, 768, 320), (512, 1536, 1024)):
        f = R.ref_fmt_new(n, subch, span)
        side = span + 30
        kind = np.zeros(side * side, np.uint8)
        R.refh_layout_kind(f, 61, oracle._p(kind))
        R.ref_fmt_free(f)
        assert np.array_equal(kind.reshape(side, side), synth.border_kind(span, synth.fmt_word(subch // 16, 61, span))), span
        cb = np.zeros(2, np.int32)
        R.refh_fmt_geometry(span, oracle._p(cb))
        assert tuple(cb) == synth.fmt_geometry(span)


def capture_cases(seed, count):
    """Seeded word captures over the three rings: clean, blurred, noisy, glare over a side (the erasure path), the
    registration's mesh off by a fraction of a pixel."""
    rng = np.random.default_rng(seed)
    out = []
    for t in range(count):
        span = SPANS[t % 3]
        pxm = (3, 2, 1)[t % 3]
        W = H = 720
        glare = None
        if t % 3 == 2 or t % 4 == 3:
            pos = [(360, 40), (680, 360), (360, 680), (40, 360)][int(rng.integers(0, 4))]
            glare = (pos[0], pos[1], float(rng.choice([80.0, 160.0, 250.0])), float(rng.choice([1.5, 3.0, 6.0])))
        luma, reg, cw = synth.word_capture(span, pxm, int(rng.integers(4, 65)), int(rng.integers(0, 256)), W, H, rng,
                                           blur=float(rng.choice([0.0, 0.8, 1.5, 2.5])), sigma=float(rng.choice([3.0, 8.0])),
                                           glare=glare, mesh=0.3 if t % 5 == 0 else 0.0)
        out.append((span, luma, reg))
    return out


def read_oracle(span, luma, reg):
    P = oracle.port()
    nodes = synth.layout_nodes(span).astype(np.float32)
    cells, nbytes = synth.fmt_geometry(span)
    q = np.zeros(4 * cells, np.float32)
    got = P.orc_fmt_read(span, oracle._p(luma), luma.shape[1], luma.shape[0], oracle._p(reg), oracle._p(nodes), nodes.size, oracle._p(q))
    vf = np.zeros(2, np.int32)
    ok = bool(got) and P.orc_fmt_decode(oracle._p(q), cells, nbytes, oracle._p(vf)) == 0
    return q, np.array([int(got > 0), int(ok), vf[0] if ok else 0, vf[1] if ok else 0], np.int32)


def test_fmt_read_matches_reference():
    """The soft values bit for bit and the word, on captures where the word reads, reads after erasures, and fails."""
    R = _ref()
    outcomes = set()
    for span, luma, reg in capture_cases(7, 36):
        q, word = read_oracle(span, luma, reg)
        cells, _ = synth.fmt_geometry(span)
        qr, wr = np.zeros(4 * cells, np.float32), np.zeros(4, np.int32)
        R.refh_fmt_read(span, oracle._p(luma), luma.shape[1], luma.shape[0], oracle._p(reg), oracle._p(qr), oracle._p(wr))
        assert np.array_equal(word, wr), (span, word, wr)
        if wr[0]:
            assert np.array_equal(q.view(np.uint32), qr.view(np.uint32)), span
        outcomes.add((int(wr[0]), int(wr[1])))
    assert {(1, 1), (1, 0)} <= outcomes, outcomes


def test_fmt_golden():
    """The oracle against the reference's outputs stored in tests/golden/fmt_ref.npz (made by make_fmt_golden.py)."""
    g = np.load(GOLDEN)
    for c in range(int(g["count"])):
        span, iw, ih = (int(v) for v in g["geom"][c])
        luma = g["luma_%d" % c].reshape(ih, iw)
        q, word = read_oracle(span, luma, g["reg_%d" % c])
        assert np.array_equal(word, g["word"][c]), c
        if word[0]:
            assert np.array_equal(q.view(np.uint32), g["q_%d" % c].view(np.uint32)), c
    P = oracle.port()
    for c in range(int(g["dcount"])):
        cells, nbytes = (int(v) for v in g["dgeom"][c])
        vf = np.zeros(2, np.int32)
        rc = P.orc_fmt_decode(oracle._p(g["dq_%d" % c]), cells, nbytes, oracle._p(vf))
        assert [rc, *(vf if rc == 0 else (0, 0))] == list(g["dout"][c]), c
