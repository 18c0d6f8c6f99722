"""End to end against the reference's own receiver: captures the reference's sender painted, decoded by the
reference's whole receiver (acquisition, then lizard_finish with its integer read, the x86-64 build) when the fixture
was made (tests/golden/make_e2e_golden.py). The GPU receiver, given the registration the reference's acquisition
held, decodes the identical set of CRC-passing blocks with the same bytes: on the plain receiver's configuration
(LIZARD-64, 1280 x 720, AWGN 2) and on distorted captures (LIZARD-1024 in 1920 x 1080, blur 0.5 and 1.5 px in linear
light, radial k1 +-0.03), where marginal blocks are decided by the last grey level's rounding."""
import lzma
import os

import numpy as np
import pytest

import lizard_gb300 as lz
import oracle

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "e2e_ref.npz")


def cases():
    z = np.load(GOLD)
    tags = sorted({k.rsplit("_", 1)[0] for k in z.files})
    out = []
    for t in tags:
        n, subch, span, w, h, x0, y0, x1, y1 = (int(v) for v in z[t + "_fmt"])
        frame = np.zeros((h, w), np.uint8)
        frame[y0:y1, x0:x1] = np.frombuffer(lzma.decompress(z[t + "_crop"].tobytes()), np.uint8).reshape(y1 - y0, x1 - x0)
        out.append((t, n, subch, span, frame, z[t + "_reg"], z[t + "_ok"], z[t + "_its"], z[t + "_blocks"]))
    return out


CASES = cases()


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_oracle_decode_read_and_blocks(case):
    """The oracle's decode read (the restatement the GPU's is held to) on the fixture's frames: its soft stage
    from its FP64 spectrum decodes the reference's verified blocks."""
    tag, n, subch, span, frame, reg, ok, its, blocks = case
    o = oracle.Fmt(n, subch, span)
    grid, _ = o.sample_decode(frame, reg)
    res = o.receive(grid)
    assert res["ok"][ok > 0].all(), "a block the reference verified failed in the oracle"


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_gpu_decodes_the_reference_crc_set(case):
    tag, n, subch, span, frame, reg, ok, its, blocks = case
    rx = lz.Receiver(n, subch, span, max_frames=2, read="decode")
    out = rx.finish_luma(np.stack([frame, frame]), np.stack([reg, reg]), grid=False)
    for k in range(2):
        assert np.array_equal(out["ok"][k], ok), "%s: CRC-pass set %s, the reference's %s" % (tag, np.nonzero(out["ok"][k])[0], np.nonzero(ok)[0])
        assert np.array_equal(out["blocks"][k][ok > 0], blocks)
    same_its = float(np.mean(out["its"][0] == its.astype(np.int32)))
    print("%s: %d of %d blocks verified as the reference; iterations equal on %.3f of the blocks" % (tag, int(ok.sum()), ok.size, same_its))
