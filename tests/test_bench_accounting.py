"""bench.py's algorithmic-byte accounting for the receiver's HBM fractions: a frame's bytes are its luma footprint
(the layout square through H, at most the frame) plus the intermediates each written and read once."""
import numpy as np

import bench
import lizard_gb300 as lz


def test_frame_bytes_of_an_axis_aligned_layout():
    fmt = lz.Format(384, 64, 128)
    side = fmt.span + 30
    s = 3.0   # pixels a module
    H = np.array([s, 0, 10, 0, s, 20, 0, 0, 1], np.float32)
    inter = 16 * fmt.n * fmt.V + 20 * 320 * fmt.subch + 480 * fmt.blocks
    # the whole layout inside a large frame: its area in pixels
    assert bench.frame_alg_bytes(fmt, H, 4000, 4000) == int((side * s) ** 2) + inter
    # a frame smaller than the layout: the footprint is the frame
    assert bench.frame_alg_bytes(fmt, H, 300, 200) == 300 * 200 + inter


def test_frame_bytes_of_a_rotated_layout_keep_its_area():
    fmt = lz.Format(768, 320, 256)
    side = fmt.span + 30
    c, sn, s = np.cos(0.3), np.sin(0.3), 2.0
    H = np.array([s * c, -s * sn, 900, s * sn, s * c, 100, 0, 0, 1], np.float64)
    inter = 16 * fmt.n * fmt.V + 20 * 320 * fmt.subch + 480 * fmt.blocks
    got = bench.frame_alg_bytes(fmt, H, 4000, 4000) - inter
    assert abs(got - (side * s) ** 2) <= 1
