"""Makes tests/golden/mesh_ref.npz: the reference's own border-node pass (refine_node over the border lattice in its
caller's order, the reference's portable build compiled from its sources into oracle/_ref/libref_scalar.so by
`make -C oracle ref`, through oracle/ref_anchor.c refs_border_nodes) on seeded captures, for the tests on machines
where the reference tree is absent. Each frame keeps only the pixels within 10 modules of the border's outer edge
(the rest set to 0), which holds every sample the pass reads; the outputs are the reference's on the stored frame.

    python tests/golden/make_mesh_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))
import oracle  # noqa: E402
from lizard_gb300_testing import synth  # noqa: E402
from test_mesh_oracle import mesh_cases  # noqa: E402


def band(span, shape, Hm):
    h, w = shape
    Hi = np.linalg.inv(Hm.astype(np.float64).reshape(3, 3))
    V, U = np.mgrid[0:h, 0:w].astype(np.float64)
    q = Hi @ np.stack([U.ravel() + 0.5, V.ravel() + 0.5, np.ones(U.size)])
    mx, my = q[0] / q[2], q[1] / q[2]
    side = span + 30
    d = np.minimum(np.minimum(mx, side - mx), np.minimum(my, side - my))
    return ((d > -3) & (d < 10)).reshape(h, w)


def main():
    R = oracle.ref_scalar()
    assert R is not None, "build the reference first: make -C oracle ref"
    out, geom, has = {}, [], []
    for c, (span, luma, Hm, lens) in enumerate(mesh_cases(17, 6)):
        kept = np.where(band(span, luma.shape, Hm), luma, 0).astype(np.uint8)
        nn = synth.layout_nodes(span).size
        nodes = np.zeros(4 * nn * nn, np.float32)
        R.refs_border_nodes(span, oracle._p(kept), kept.shape[1], kept.shape[0], oracle._p(Hm), None if lens is None else oracle._p(lens), oracle._p(nodes))
        out["luma_%d" % c], out["H_%d" % c], out["nodes_%d" % c] = kept.ravel(), Hm, nodes
        out["lens_%d" % c] = lens if lens is not None else np.zeros(15)
        geom.append((span, kept.shape[1], kept.shape[0]))
        has.append(lens is not None)
    out["count"], out["geom"], out["has_lens"] = np.int32(len(geom)), np.array(geom, np.int32), np.array(has, bool)
    path = os.path.join(ROOT, "tests", "golden", "mesh_ref.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
