"""Makes tests/golden/encode_ref.npz: crops of the reference sender's own grey pages (lizard_encode +
lizard_paint_grey, compiled from the reference's sources into oracle/_ref/libref.so by `make -C oracle ref`), for the
tests on machines where the reference tree is absent. Cases: LIZARD-64 in the 64 ring (exact copy, 3 pixels a
module) and in the 128 ring (resampled, 2 pixels a module), seeded blocks (lizard_gb300.synth.random_blocks), pilot
counts 1 and 2. Each page keeps its top-left corner and the square about its middle anchor.

    python tests/golden/make_encode_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))
import lizard_gb300 as lz  # noqa: E402
from lizard_gb300_testing import synth  # noqa: E402
from test_encode_oracle import _ref, golden_crops, ref_page  # noqa: E402


def main():
    R = _ref()
    out, cases = {}, []
    for c, (n, subch, span, seed, pilots) in enumerate(((384, 64, 128, 11, 1), (384, 64, 256, 12, 2))):
        fmt = lz.Format(n, subch, span)
        _, grey = ref_page(R, n, subch, span, synth.random_blocks(fmt.blocks, seed), pilots)
        for k, crop in enumerate(golden_crops(grey, synth.pxm_for(n, span))):
            out["crop_%d_%d" % (c, k)] = crop
        cases.append((n, subch, span, seed, pilots))
    out["count"] = np.int32(len(cases))
    out["case"] = np.array(cases, np.int32)
    path = os.path.join(ROOT, "tests", "golden", "encode_ref.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
