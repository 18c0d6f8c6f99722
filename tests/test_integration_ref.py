"""The reference-side integration compiles and runs: lizard_gb300/integration/lizard_finish_gpu.c (lizard_finish on
the GPU for the reference's own codec) and a check program, compiled against the reference's own headers and linked
with its objects and liblizard_gb300.so (oracle/Makefile's `integration` target, where the reference tree is present).
The program registers a frame with the reference's lizard_acquire, finishes it on the GPU, finishes it again with the
reference's lizard_finish and compares. Without a GPU it stops where the library reports no device (no fallback)."""
import os
import subprocess
import sys

import numpy as np
import pytest

import oracle
from conftest import ROOT, gpu_available

pytestmark = pytest.mark.skipif(not oracle.have_ref(), reason="the reference is not built here")


def test_glue_compiles_links_and_runs(tmp_path):
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "integration", "LIZARD_REF=" + oracle.REF_ROOT], check=True)
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    from make_e2e_golden import case_c1
    r, span, luma = case_c1(0)
    raw = tmp_path / "frame.raw"
    raw.write_bytes(np.array(luma.shape[::-1], np.int32).tobytes() + luma.tobytes())
    p = subprocess.run([os.path.join(ROOT, "oracle", "_ref", "finish_gpu_check"), str(raw), "384", "64", "128"], capture_output=True, text=True, timeout=300)
    if gpu_available():
        assert p.returncode == 0, p.stdout + p.stderr
        assert "same 1" in p.stdout
    else:
        assert p.returncode == 3, p.stdout + p.stderr
        assert p.stdout.startswith("nogpu:") and len(p.stdout.strip()) > len("nogpu:")
