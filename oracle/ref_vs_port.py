"""Times the reference's own LDPC decoder (ldpc_decode_stall compiled from its sources, oracle/_ref: the x86-64 build
with its SSE4.1 / AVX2 layers) against the oracle's plain-C restatement (oracle/_build) on the same mixed-rate batch
and thread count, and checks their outputs identical. TEST AND MEASUREMENT INFRASTRUCTURE ONLY: the GPU host has no
reference tree, so its CPU baseline runs the restatement; this factor converts that figure into the reference's.

Run from the repo root where the reference is present: python oracle/ref_vs_port.py  (writes oracle/ref_vs_port.json)
"""
import json
import os
import platform
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
import oracle  # noqa: E402
from lizard_gb300_testing import synth  # noqa: E402

COUNT, MAX_ITER, STALL_IT, STALL_RATIO = 16384, 20, 9, 0.95


def timed(lib, b, threads, reps=3):
    best, out = None, None
    for _ in range(reps):
        t0 = time.perf_counter()
        out = oracle.ldpc_batch(lib, b["llr"], b["offsets"], b["rates"], MAX_ITER, STALL_IT, STALL_RATIO, threads=threads)
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    return best, out


def main():
    oracle.build(ref=True)
    if not oracle.have_ref():
        raise SystemExit("the reference is not built here")
    b = synth.ldpc_batch(COUNT, seed=1000)
    res = {"workload": "%d codewords of the benchmark batch (seed 1000: 39/26/15/20%% 7/8,3/4,2/3,1/2, Eb/N0 1.0-4.0 dB), "
                       "max %d iterations, stall %d/%.2f" % (COUNT, MAX_ITER, STALL_IT, STALL_RATIO),
           "host": {"machine": platform.machine(), "processor": platform.processor() or None, "threads_available": os.cpu_count()},
           "reference_build": "liblizard/src compiled with -O3 -ffp-contract=off -march=x86-64-v2 (run-time AVX2 layers)",
           "port_build": "oracle/*.c with -O3 -ffp-contract=off (gcc's own vectorisation)", "runs": []}
    for threads in sorted({1, os.cpu_count() or 1}):
        tr, (rb, ri, ro) = timed(oracle.ref(), b, threads)
        tp, (pb, pi, po) = timed(oracle.port(), b, threads)
        assert np.array_equal(rb, pb) and np.array_equal(ri, pi) and np.array_equal(ro, po), "the restatement differs from the reference"
        res["runs"].append({"threads": threads, "reference_s": round(tr, 3), "port_s": round(tp, 3),
                            "reference_Gbps": round(COUNT * 3840 / tr / 1e9, 4), "port_Gbps": round(COUNT * 3840 / tp / 1e9, 4),
                            "reference_over_port": round(tp / tr, 3), "identical_outputs": True})
    res["reference_over_port"] = res["runs"][-1]["reference_over_port"]
    path = os.path.join(HERE, "ref_vs_port.json")
    with open(path, "w") as f:
        json.dump(res, f, indent=1)
    print(json.dumps(res, indent=1))


if __name__ == "__main__":
    main()
