#!/usr/bin/env python
"""Benchmark: LIZARD's LDPC decoder batch on one GB300 (decoded information Gbit/s).

Workload: 65,536 codewords of the four codes in the format's proportions (39% 7/8, 26% 3/4, 15% 2/3, 20% 1/2 by
count), each a 476-byte block plus its CRC-32C, BPSK over AWGN with Eb/N0 cycling 1.0 to 4.0 dB in 0.5 dB steps,
quantised to the reference's int8 soft values; layered min-sum, at most 20 iterations, the stall rule (9, 0.95),
then the CRC-32C check. One step decodes the whole batch (its LLRs, ~354 MB, are larger than L2, so no flush is
needed between steps).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line. `value` is device-timed with the LLRs resident in HBM; `e2e` is the same metric through the
C ABI's host-memory entry point (pinned host buffers, copies in and out inside the timed region). The CPU baseline
times the reference's CPU decoder (compiled from its sources where present, else the oracle's C restatement) on the
same batch on the host's cores.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "decoded payload MB/s, frames/s and LDPC Gbit/s on 1 GB300, refined+batched vs plain"
UNIT = "Gbit/s"
MAX_ITER, STALL_IT, STALL_RATIO = 20, 9, 0.95


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--count", type=int, default=65536, help="codewords a step (the workload: 65,536)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-receiver", action="store_true", help="skip the frame receiver's workloads")
    ap.add_argument("--receiver-only", action="store_true", help="time only the frame receiver (profiling)")
    ap.add_argument("--no-autotune", action="store_true", help="keep the decoder's default kernel variants")
    ap.add_argument("--batch-only", action="store_true", help="with --receiver-only: only the batched workloads (FFT demod batch, "
                    "anchor search), for profiling")
    ap.add_argument("--ingest-only", action="store_true", help="time only the camera-format ingest (profiling)")
    ap.add_argument("--fmt-only", action="store_true", help="time only the format word and the border nodes (profiling)")
    ap.add_argument("--encode-only", action="store_true", help="time only the sender on the GPU (profiling)")
    ap.add_argument("--refine-only", action="store_true", help="time only the distorted captures' registration comparison")
    ap.add_argument("--multistream-only", action="store_true", help="time only the multi-stream tick (profiling)")
    ap.add_argument("--refine-frames", type=int, default=0, help="with --refine-only: the first K frames of the spread set alone "
                    "(profiling; 0: the configuration's three sets)")
    ap.add_argument("--ldpc-variants", action="store_true", help="time every decoder kernel variant of every code on the "
                    "workload's codewords of that code (device-resident), outputs checked identical across variants")
    return ap.parse_args()


def workload(count):
    return {"workload": "LDPC decoder batch: %d codewords, 39/26/15/20%% 7/8,3/4,2/3,1/2, BPSK/AWGN Eb/N0 1.0-4.0 dB "
                        "(0.5 dB steps, cycled), int8 LLRs, layered min-sum max %d its, stall %d/%.2f, CRC-32C" % (count, MAX_ITER, STALL_IT, STALL_RATIO),
            "codewords": count, "info_bits_per_codeword": 3840, "max_iter": MAX_ITER, "stall": [STALL_IT, STALL_RATIO],
            "l2": "inputs larger than L2 (no flush)", "parallelism": "replicas (codewords independent)"}


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, 0
    import torch
    import torch.distributed as dist
    rank, local = int(os.environ["RANK"]), int(os.environ.get("LOCAL_RANK", "0"))
    if torch.cuda.is_available():
        torch.cuda.set_device(local)
    dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return rank, ws, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, ws):
    if ws <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 100 ms while running."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device, self.p, self.path = device, None, None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(prefix="lizg_clocks_", suffix=".csv")
            self.f = os.fdopen(fd, "w")
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                       "-lms", "100"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()
            self.f.close()

    def summary(self):
        if not self.p or not self.path:
            return None
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        try:
            os.remove(self.path)   # the summary is what the result line carries
        except OSError:
            pass
        self.path = None
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, flags in rows for i, v in enumerate(flags) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


def peaks():
    try:
        d = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(d["hbm_gbs"]), "of measured"
    except Exception:
        return 6800.0, "of fallback"


def traffic_per_step(count):
    """DRAM bytes per step from the committed ncu summary (profiles/ldpc_traffic.json), scaled to `count` codewords."""
    try:
        d = json.load(open(os.path.join(ROOT, "profiles", "ldpc_traffic.json")))
        return float(d["dram_bytes_per_codeword"]) * count
    except Exception:
        return None


def cpu_decode(batch, threads, sample, outputs=False):
    """The CPU decoder on the first `sample` codewords: (Gbit/s, seconds, kind), and with outputs its (packed bits,
    its, ok)."""
    import numpy as np
    import oracle
    lib, kind = (oracle.ref(), "reference") if oracle.have_ref() else (oracle.port(), "port")
    n = int(batch["offsets"][sample - 1]) + {6: 4608, 4: 5120, 3: 5760, 2: 7680}[int(batch["rates"][sample - 1])] if sample < batch["rates"].size else batch["llr"].size
    t0 = time.perf_counter()
    out = oracle.ldpc_batch(lib, batch["llr"][:n], batch["offsets"][:sample], batch["rates"][:sample], MAX_ITER, STALL_IT, STALL_RATIO, threads=threads)
    dt = time.perf_counter() - t0
    if outputs:
        return sample * 3840 / dt / 1e9, dt, kind, out
    return sample * 3840 / dt / 1e9, dt, kind


def ref_over_port():
    """The reference decoder's speed over the restatement's on one host (oracle/ref_vs_port.json, measured where the
    reference compiles), or None."""
    try:
        d = json.load(open(os.path.join(ROOT, "oracle", "ref_vs_port.json")))
        return float(d["reference_over_port"]), d["host"]["machine"], d["runs"][-1]["threads"]
    except Exception:
        return None


def reference_estimate(value, kind):
    """A restatement's figure converted to the reference decoder's by the factor measured where both run."""
    f = ref_over_port()
    if kind != "port" or f is None:
        return None
    return {"value": round(value * f[0], 4), "unit": UNIT, "factor": f[0],
            "source": "oracle/ref_vs_port.json: the reference's own ldpc_decode_stall (its SIMD layers) over the restatement, "
                      "same batch, %d threads of an %s host; the GPU host (aarch64) has no reference tree to time it there" % (f[2], f[1]),
            "measured": False}


# Integer operations an edge update costs at the least in layered min-sum (liblizard/src/ldpc.c:141-192): the extrinsic
# q = L - R, its saturation to 8 bits, |q|, the running min1 / min2 (two min/max), the sign's XOR, the message's
# sign select, the posterior L = q + R.
OPS_PER_EDGE = 8
ALU_LANES_PER_SM = 64   # 4 sub-partitions x 16 lanes: one ALU warp-instruction every 2 cycles each


def int_op_roofline(edges, launch_ms, sm_mhz, sms):
    """The decoder's integer roofline from this run: edge updates a second x OPS_PER_EDGE against the ALU pipe's
    peak at the run's median SM clock."""
    if not sm_mhz:
        return None
    achieved = edges / (launch_ms / 1e3) * OPS_PER_EDGE / 1e12
    peak = sms * ALU_LANES_PER_SM * sm_mhz * 1e6 / 1e12
    return {"achieved": round(achieved, 3), "peak": round(peak, 3), "unit": "Tops/s", "frac": round(achieved / peak, 4),
            "ops_per_edge_update": OPS_PER_EDGE, "peak_from": "%d SMs x %d ALU lanes x the median SM clock under load (%.0f MHz)" % (sms, ALU_LANES_PER_SM, sm_mhz)}


def picture_frames(fmt, count, seed, sigma):
    """count distinct pictures painted by the sender (the library's GPU encoder at the 64 ring's exact-copy scale, so
    the picture's region of the page is the picture itself), each seeded blocks, AWGN of sigma grey levels: luma frames
    of the picture alone (w = h = n) on the device, and the registration that samples them one pixel a sample."""
    import numpy as np
    import torch
    import lizard_gb300 as lz
    from lizard_gb300_testing import render, synth
    n, scale = fmt.n, fmt.n / fmt.span
    nn = synth.layout_nodes(fmt.span).size
    reg = np.concatenate([np.array([scale, 0, -15 * scale, 0, scale, -15 * scale, 0, 0, 1], np.float32), np.zeros(2 * nn * nn, np.float32)])
    blocks = np.stack([synth.random_blocks(fmt.blocks, seed * 1000 + u) for u in range(count)])
    pg, pxm = render.pages(lz, n, fmt.subch, fmt.span, blocks, 1)
    assert pxm * fmt.span == n, "an exact-copy scale"
    o = (render.QUIET + 15) * pxm
    gen = torch.Generator(device="cuda")
    gen.manual_seed(seed)
    pic = pg[:, o:o + n, o:o + n].to(torch.float32)
    luma = torch.clamp(torch.round(pic + sigma * torch.randn(pic.shape, generator=gen, device="cuda")), 0, 255).to(torch.uint8)
    return luma.contiguous(), np.tile(reg, (count, 1))


def fft_error_table():
    """The transform's error per picture size on the FFT demod batch's sizes (n = 384, 768, 1152, 1536 at their top
    versions): the GPU's spectrum against the reference's own FP32 one (tests/golden/fft_ref.npz, made by the reference
    compiled from its sources; every eighth coefficient) and against the FP64 oracle (every coefficient), max and rms
    relative to the spectrum's rms; the reference's own FP32 against FP64 beside them."""
    import hashlib
    import numpy as np
    import lizard_gb300 as lz
    import oracle
    from lizard_gb300_testing import synth
    if not os.path.exists(oracle.PORT_PATH):
        oracle.build(ref=False)
    z = np.load(os.path.join(ROOT, "tests", "golden", "fft_ref.npz"))
    table = {}
    for n in (384, 768, 1152, 1536):
        n_, subch, span = (int(v) for v in z["n%d_fmt" % n])
        f = lz.Format(n_, subch, span)
        g, _ = synth.grids(f, 1, seed=31 * n, sigma=3.0, shift=(0.15, -0.1))
        if hashlib.sha256(np.rint(g[0] * 255.0).astype(np.uint8).tobytes()).digest() != z["n%d_sha256" % n].tobytes():
            table[n] = {"error": "the grid made here differs from the fixture's"}
            continue
        c = lz.Receiver(n_, subch, span, max_frames=1).finish_grid(g)["coef"][0]
        c = c[0::2] + 1j * c[1::2]
        r = z["n%d_ref" % n]
        ref = r[:, 0].astype(np.float64) + 1j * r[:, 1]
        fp64, _, _ = oracle.Fmt(n_, subch, span).spectrum(g[0])
        idx = np.arange(0, c.size, 8)

        def err(a, b):
            rms = np.sqrt(np.mean(np.abs(b) ** 2))
            e = np.abs(a - b)
            return {"max": float("%.3g" % (e.max() / rms)), "rms": float("%.3g" % (np.sqrt(np.mean(e ** 2)) / rms))}
        table[n] = {"vs_reference_fp32": err(c[idx], ref), "vs_fp64": err(c, fp64), "reference_fp32_vs_fp64": err(ref, fp64[idx]),
                    "bar": 1e-4}
    return table


def bench_receiver(args, stream):
    """The frame receiver, rows a-e (sampler, erase, detrend, 2D FFT, pilots, demap, LDPC, CRC), on two workloads:
    the FFT demod batch (256 pictures: 64 each at n = 384, 768, 1152, 1536 at their top versions, 64 ring, AWGN 3
    grey levels, one call per picture size) and the plain receiver one frame a call (LIZARD-64, n = 384, 1280 x 720,
    AWGN 2). Device-timed with CUDA events; frames/s and payload MB/s (472 bytes a verified block)."""
    import numpy as np
    import torch
    import lizard_gb300 as lz
    from lizard_gb300_testing import synth
    res = {}
    sp = stream.cuda_stream
    # --- FFT demod batch
    sizes = [(384, 80), (768, 320), (1152, 720), (1536, 1024)]
    per = 64
    rxs, bufs, blocks_total, step_bytes = [], [], 0, 0
    for n, subch in sizes:
        rx = lz.Receiver(n, subch, 128, max_frames=per)
        d_l, reg = picture_frames(rx.fmt, per, seed=n, sigma=3.0)
        step_bytes += per * frame_alg_bytes(rx.fmt, reg[0], n, n)
        d_r = torch.from_numpy(reg).cuda()
        o, s = rx._outputs(per, torch, keep=False)
        rxs.append(rx)
        bufs.append((d_l, d_r, o, s, n))
        blocks_total += per * rx.fmt.blocks

    def step():
        for rx, (d_l, d_r, o, s, n) in zip(rxs, bufs):
            lz._check(lz.lib().lizg_rx_finish_luma_dev(rx._h, lz.ctypes.c_void_p(d_l.data_ptr()), n, n, n, n * n, lz.ctypes.c_void_p(d_r.data_ptr()),
                                                         per, lz.ctypes.byref(s), None, None, lz.ctypes.c_void_p(sp)), "finish_luma")

    K = max(1, args.steps // 3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed():
        for _ in range(max(args.warmup, 3)):
            step()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(K):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / K

    # the device's LDPC variants (tuned on large batches of one code), then each handle's own per-tier choice timed
    # on its batch (lizg_rx_autotune: per picture size and code rate)
    ms_global = timed()
    ok_global = [b[2]["ok"].clone() for b in bufs]
    choices = {}
    for rx, (d_l, d_r, o, s, n) in zip(rxs, bufs):
        v = rx.autotune_dev(d_l.data_ptr(), n, n, n, n * n, d_r.data_ptr(), per, sp)[:rx.fmt.tiers]
        mixed = rx.set_ldpc_mixed(0)
        rx.set_ldpc_mixed(mixed)
        choices[str(n)] = {"variants": v, "one_launch_across_tiers": bool(mixed)}
    ms = timed()
    ok = sum(int(b[2]["ok"].sum().item()) for b in bufs)
    same = all(bool(torch.equal(a, b[2]["ok"])) for a, b in zip(ok_global, bufs))
    res["fft_demod_batch"] = {"workload": "256 distinct pictures, 64 each at n=384/768/1152/1536 (LIZARD-80/320/720/1024), 64 ring, painted by the sender, "
                                          "AWGN 3 DN, rows a-e, one call per size",
                              "frames_per_s": round(256 / (ms / 1e3), 1), "payload_MBps": round(ok * 472 / (ms / 1e3) / 1e6, 2),
                              "ms_per_step": round(ms, 3), "blocks_verified": ok, "blocks": blocks_total,
                              "gpu_launches_per_step": sum(rx.launches for rx in rxs),
                              "ldpc_per_n_and_rate": {"per_n": choices, "frames_per_s_device_choice": round(256 / (ms_global / 1e3), 1),
                                                      "identical_verdicts": same}}
    peak, peak_src = peaks()
    res["fft_demod_batch"]["error_per_n"] = fft_error_table()
    res["fft_demod_batch"]["hbm"] = {"algorithmic_bytes_per_step": step_bytes, "GBps": round(step_bytes / (ms / 1e3) / 1e9, 1),
                                     "frac": round(step_bytes / (ms / 1e3) / 1e9 / peak, 4), "peak_source": peak_src,
                                     "bytes": "luma footprint + Y written and read + used coefficients and soft values written and read + blocks"}
    # --- one frame a call (direct and captured), and a batch of frames a call, at n = 384 and n = 1536
    def capture_frames(n, subch, W, Hh, count, seed):
        rx = lz.Receiver(n, subch, 128, max_frames=count)
        rng = np.random.default_rng(seed)
        lumas, regs = [], []
        for u in range(min(count, 4)):
            grey = synth.picture(rx.fmt, synth.random_blocks(rx.fmt.blocks, seed + u), parity=u & 3)
            luma, reg = synth.capture(rx.fmt, grey, W, Hh, sigma=2.0, rng=rng)
            lumas.append(luma)
            regs.append(reg)
        luma = np.stack([lumas[i % len(lumas)] for i in range(count)])
        reg = np.stack([regs[i % len(regs)] for i in range(count)])
        return rx, torch.from_numpy(luma).cuda(), torch.from_numpy(reg).cuda()

    def timed(call, K):
        for _ in range(10):
            call()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(K):
            call()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / K

    def receiver_line(n, subch, W, Hh, frames, graph, K, label, tune=False):
        rx, d_l, d_r = capture_frames(n, subch, W, Hh, frames, seed=n)
        o, s = rx._outputs(frames, torch, keep=False)
        choice = None
        if tune:   # the handle's own decode: each tier's variant and one launch across the tiers or a launch a tier
            choice = rx.autotune_dev(d_l.data_ptr(), W, Hh, W, W * Hh, d_r.data_ptr(), frames, sp)[:rx.fmt.tiers]
            mixed = rx.set_ldpc_mixed(0)
            rx.set_ldpc_mixed(mixed)
        fn = lz.lib().lizg_rx_finish_luma_graph if graph else lz.lib().lizg_rx_finish_luma_dev

        def call():
            lz._check(fn(rx._h, lz.ctypes.c_void_p(d_l.data_ptr()), W, Hh, W, W * Hh, lz.ctypes.c_void_p(d_r.data_ptr()), frames,
                         lz.ctypes.byref(s), None, None, lz.ctypes.c_void_p(sp)), "finish_luma")
        ms = timed(call, K)
        okb = int(o["ok"].sum().item())
        line = {"workload": label, "frames_per_call": frames, "graph": graph, "frames_per_s": round(frames / (ms / 1e3), 1),
                "payload_MBps": round(okb * 472 / (ms / 1e3) / 1e6, 3), "ms_per_call": round(ms, 4),
                "blocks_verified": okb, "blocks": frames * rx.fmt.blocks, "gpu_launches_per_call": rx.launches}
        if tune:
            line["ldpc_decode"] = {"variants_per_tier": choice, "one_launch_across_tiers": bool(mixed)}
        return line

    if args.batch_only:
        return res
    res["plain_one_frame"] = receiver_line(384, 64, 1280, 720, 1, False, 200, "LIZARD-64, n=384, 64 ring, 1280x720 luma, AWGN 2 DN, axis-aligned, one frame a call")
    res["plain_one_frame_graph"] = receiver_line(384, 64, 1280, 720, 1, True, 400, "the same, the call replayed from a CUDA graph")
    res["plain_one_frame_graph_tuned"] = receiver_line(384, 64, 1280, 720, 1, True, 400, "the same from a graph, the handle's decode "
                                                       "tuned on the frame (lizg_rx_autotune)", tune=True)
    res["n1536_one_frame"] = receiver_line(1536, 1024, 3840, 2160, 1, False, 50, "LIZARD-1024, n=1536, 64 ring, 3840x2160 luma, AWGN 2 DN, one frame a call")
    res["n1536_batched_graph"] = receiver_line(1536, 1024, 3840, 2160, 32, True, 5, "the same, 32 frames a call replayed from a CUDA graph")
    res["n1536_batched_vs_one_frame"] = round(res["n1536_batched_graph"]["frames_per_s"] / res["n1536_one_frame"]["frames_per_s"], 2)
    res["n1536_batched_refined"] = batched_refined_line(rx_frames=capture_frames, timed=timed, stream=stream, one_frame=res["n1536_one_frame"])
    return res


def batched_refined_line(rx_frames, timed, stream, one_frame):
    """Batched and refined against the plain receiver one frame a launch, at n = 1536 on clean inputs (the same
    frames as n1536_one_frame): 32 frames a call decoded, the frames the decode left blocks unverified in refined by
    the adjoint refinement (lizg_field_refine_dev, gated on them; anchors measured through the registration) and
    decoded again. Also the refinement's cost with the gate open on every frame (the outputs then checked
    unchanged: a registration already right stays right)."""
    import torch
    import lizard_gb300 as lz
    frames, W, Hh = 32, 3840, 2160
    rx, d_l, d_r = rx_frames(1536, 1024, W, Hh, frames, seed=1536)
    fmt = rx.fmt
    sp = stream.cuda_stream
    stride = d_r.shape[1]
    d_g = torch.empty_like(d_r)
    o, s = rx._outputs(frames, torch, keep=False)
    o0, s0 = rx._outputs(frames, torch, keep=False)
    d_gate = torch.zeros(frames, dtype=torch.uint8, device="cuda")
    ao = {"ok": torch.zeros((frames, 49), dtype=torch.uint8, device="cuda")}
    for key in ("peak", "dx", "dy", "u", "v"):
        ao[key] = torch.zeros((frames, 49), dtype=torch.float32, device="cuda")
    a_out = lz.AnchorOut(*[ao[key].data_ptr() for key in ("ok", "peak", "dx", "dy", "u", "v")])
    fld = lz.FieldRefiner(1536, 1024, 128, chunk=32)

    def finish(d_reg, so):
        lz._check(lz.lib().lizg_rx_finish_luma_dev(rx._h, lz.ctypes.c_void_p(d_l.data_ptr()), W, Hh, W, W * Hh, lz.ctypes.c_void_p(d_reg.data_ptr()),
                                                   frames, lz.ctypes.byref(so), None, None, lz.ctypes.c_void_p(sp)), "finish_luma")

    def call(force=False):
        d_g.copy_(d_r)
        finish(d_g, s)
        if force:
            d_gate.fill_(1)
        else:
            d_gate.copy_((o["ok"].sum(dim=1) < fmt.blocks).to(torch.uint8))
            if not bool(d_gate.any().item()):   # every frame verified: nothing to refine
                return
        lz._check(lz.lib().lizg_anchor_find_dev(128, lz.ctypes.c_void_p(d_l.data_ptr()), W, Hh, W * Hh, lz.ctypes.c_void_p(d_g.data_ptr()), stride,
                                                None, None, frames, lz.ctypes.byref(a_out), lz.ctypes.c_void_p(sp)), "anchor_find")
        fld.refine_dev(d_l.data_ptr(), W, Hh, W * Hh, d_g.data_ptr(), frames, 3, a_out, d_gate.data_ptr(), None, None, sp)
        finish(d_g, s)

    finish(d_r, s0)   # the plain registration's outputs, to compare
    ms = timed(call, 10)
    same = bool(torch.equal(o["ok"], o0["ok"]) and torch.equal(o["its"], o0["its"]) and torch.equal(o["blocks"], o0["blocks"]))
    refined = int(d_gate.sum().item())
    ms_forced = timed(lambda: call(True), 3)
    same_forced = bool(torch.equal(o["ok"], o0["ok"]))
    fld.close()
    fps = frames / (ms / 1e3)
    return {"workload": "LIZARD-1024, n=1536, 3840x2160 clean captures (as n1536_one_frame), 32 frames a call: decode, the frames with "
                        "unverified blocks refined by the adjoint refinement (3 steps, anchors measured) and decoded again",
            "frames_per_s": round(fps, 1), "ms_per_call": round(ms, 4), "frames_refined": refined,
            "vs_plain_one_frame_a_launch": round(fps / one_frame["frames_per_s"], 2), "identical_decoded_output": same,
            "gate_open_on_every_frame": {"frames_per_s": round(frames / (ms_forced / 1e3), 1), "ms_per_call": round(ms_forced, 4),
                                         "identical_crc_sets": same_forced}}


def warped_frames(n, subch, span, W, Hh, count, seed0, scale):
    """count distinct captures (W x Hh luma on the device): seeded blocks painted by the sender (the library's GPU
    encoder, the page with its border), each under its own warp (synth.warp: rotation up to 15 degrees, a little
    perspective, scale x the page's pixels a module), AWGN 3 DN, rendered on the GPU. Also the warps (3 x 3 each)."""
    import numpy as np
    import torch
    import lizard_gb300 as lz
    from lizard_gb300_testing import render, synth
    fmt = lz.Format(n, subch, span)
    blocks = np.stack([synth.random_blocks(fmt.blocks, seed0 + k) for k in range(count)])
    pg, pxm = render.pages(lz, n, subch, span, blocks, 1)
    d_l = torch.empty((count, Hh, W), dtype=torch.uint8, device="cuda")
    Hws = []
    for k in range(count):
        rng = np.random.default_rng(seed0 + k)
        Hw = np.asarray(synth.warp(fmt, W, Hh, rng, rot_deg=15, scale=scale), np.float64).reshape(3, 3)
        d_l[k] = render.capture(pg[k], pxm, W, Hh, Hw, 0.0, 0.0, 3.0, seed0 + k)
        Hws.append(Hw)
    return d_l, Hws


def bench_anchor(args, stream):
    """The registration assist: the 7 x 7 anchor search (lizg_anchor_find_dev) on a batch of 64 captured 1920 x 1080
    frames, each one LIZARD-1024 symbol (n = 1536) in the 128 ring at about 2.6 pixels a module, rotated up to 15
    degrees, its map H put up to a module off. Device-timed with CUDA events; beside it the same search's arithmetic
    on the host cores (the oracle's restatement of the reference's portable build, one frame a thread)."""
    import concurrent.futures
    import numpy as np
    import torch
    import lizard_gb300 as lz
    from lizard_gb300_testing import synth
    import oracle
    span, n, subch, W, Hh, frames = 256, 1536, 1024, 1920, 1080, 64
    d_l, Hws = warped_frames(n, subch, span, W, Hh, frames, 500, (0.42, 0.45))
    lumas = list(d_l.cpu().numpy())
    Hs = []
    for k in range(frames):
        rng = np.random.default_rng(10500 + k)
        H = (Hws[k] / Hws[k][2, 2]).astype(np.float32).ravel()
        H[2] += np.float32(rng.uniform(-1, 1) * 2.6)
        H[5] += np.float32(rng.uniform(-1, 1) * 2.6)
        Hs.append(H)
    Hf = np.stack(Hs).astype(np.float32)
    d_h = torch.from_numpy(Hf).cuda()
    o = {"ok": torch.zeros((frames, 49), dtype=torch.uint8, device="cuda")}
    for key in ("peak", "dx", "dy", "u", "v"):
        o[key] = torch.zeros((frames, 49), dtype=torch.float32, device="cuda")
    s = lz.AnchorOut(*[o[key].data_ptr() for key in ("ok", "peak", "dx", "dy", "u", "v")])
    sp = stream.cuda_stream

    def call():
        lz._check(lz.lib().lizg_anchor_find_dev(span, lz.ctypes.c_void_p(d_l.data_ptr()), W, Hh, W * Hh, lz.ctypes.c_void_p(d_h.data_ptr()), 9,
                                                None, None, frames, lz.ctypes.byref(s), lz.ctypes.c_void_p(sp)), "anchor_find")
    for _ in range(3):
        call()
    torch.cuda.synchronize()
    reps = max(5, args.steps // 3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        call()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    found = int(o["ok"].sum().item())
    # the host cores: the same search's arithmetic (the oracle's plain C), one frame a thread, every frame once
    if not os.path.exists(oracle.PORT_PATH):
        oracle.build(ref=False)
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    with concurrent.futures.ThreadPoolExecutor(threads) as ex:
        cpu = list(ex.map(lambda k: oracle.anchor_find(oracle.port(), "orc_anchor_find", span, lumas[k], Hs[k]), range(frames)))
    dt = time.perf_counter() - t0
    same = all(np.array_equal(cpu[k]["ok"], o["ok"][k].cpu().numpy()) and np.array_equal(cpu[k]["dx"], o["dx"][k].cpu().numpy()) for k in range(frames))
    return {"workload": "anchor search, 64 distinct frames of 1920x1080, LIZARD-1024 (n=1536) in the 128 ring painted by the sender at ~2.6 px a module, "
                        "rotation up to 15 deg, H up to a module off, AWGN 3 DN",
            "frames_per_s": round(frames / (ms / 1e3), 1), "anchors_per_s": round(49 * frames / (ms / 1e3), 1), "ms_per_call": round(ms, 4),
            "anchors_found": found, "anchors": 49 * frames, "gpu_launches_per_call": 1, "identical_to_host": bool(same),
            "cpu": {"frames_per_s": round(frames / dt, 1), "cores": threads, "kind": "port",
                    "sample": "the 64 frames once, one frame a thread (%.2f s wall)" % dt}}


def frame_alg_bytes(fmt, H, w, h):
    """A frame's algorithmic bytes through rows a-e on the fused path (each stage's inputs read once, outputs written
    once): the luma footprint (the layout square's area through H, a byte a pixel, at most the w x h frame), the column transforms' kept rows Y
    written and read (8 n V B each way), the used coefficients written and read (8 B each way), their soft values
    written and read (2 B a coefficient each way), and the decoded blocks (476 bytes, its and ok: 480 B a block)."""
    import numpy as np
    side = fmt.span + 30
    c = np.array([[0, 0, 1], [side, 0, 1], [side, side, 1], [0, side, 1]], np.float64)
    q = c @ np.asarray(H[:9], np.float64).reshape(3, 3).T
    x, y = q[:, 0] / q[:, 2], q[:, 1] / q[:, 2]
    area = 0.5 * abs(np.dot(x, np.roll(y, -1)) - np.dot(y, np.roll(x, -1)))
    used = 320 * fmt.subch
    return int(min(area, w * h)) + 16 * fmt.n * fmt.V + 16 * used + 4 * used + 480 * fmt.blocks


def bench_multistream(args, stream):
    """Batched multi-stream decode with device registration: 32 camera streams of 3840 x 2160 luma at a nominal 60
    frames/s, picture sizes uneven across 384-1536 and rings mixed 64 / 128 / 256 (five formats; 10, 8, 6, 5 and 3
    streams), each stream's frame painted by the sender and seen as the distorted full receiver's frames are (rotation
    U(+-15 deg), tilt U(+-20 deg), the layout's side 1700 px x U(0.8, 1.1), radial k1 U(+-0.05), blur U(0.5, 2.0) px in
    linear light, AWGN 3 DN), registered from a finder's corners. A tick (one frame of every stream): the anchors'
    registration (3 rounds of the anchor search and the lens model, lizg_refine_dev) one batch a format, each format on
    its own stream, then the multi-stream engine: one receiver batch a format, each on its own stream from its own CUDA
    graph. Beside it the same
    frames one frame a launch (lizg_refine_dev and lizg_rx_finish_luma_dev a frame). Device-timed; the two paths'
    CRC-passing block sets are checked identical."""
    import numpy as np
    import torch
    import lizard_gb300 as lz
    from lizard_gb300_testing import render, synth
    W, Hh = 3840, 2160
    formats = [(384, 64, 128, 10), (768, 320, 128, 8), (1152, 720, 256, 6), (1536, 1024, 256, 5), (1536, 1024, 512, 3)]
    eng = lz.Engine()
    sp = stream.cuda_stream
    batches, keep, singles = [], [], []
    tick_bytes = 0
    rng = np.random.default_rng(700)
    for i, (n, subch, span, count) in enumerate(formats):
        eng.add_format(n, subch, span, count)
        fmt = eng.formats[i]
        seeds = [7000 + 100 * i + k for k in range(count)]
        dist = [(float(rng.uniform(-0.05, 0.05)), float(rng.uniform(0.5, 2.0))) for _ in range(count)]
        vs = render.views(n, span, W, Hh, seeds, 1700.0)
        pg, pxm = render.pages(lz, n, subch, span, np.stack([synth.random_blocks(fmt.blocks, s) for s in seeds]), 1)
        d_l = torch.empty((count, Hh, W), dtype=torch.uint8, device="cuda")
        for k in range(count):
            d_l[k] = render.capture(pg[k], pxm, W, Hh, vs[k], dist[k][0], dist[k][1], 3.0, seeds[k])
        del pg
        plain = np.stack([render.registration(span, vs[k], dist[k][0], W, Hh) for k in range(count)])
        tick_bytes += sum(frame_alg_bytes(fmt, plain[k], W, Hh) for k in range(count))
        d_p = torch.from_numpy(plain).cuda()
        d_r = torch.empty_like(d_p)
        o, so = lz.rx_outputs(fmt, count)
        refiner = lz.Refiner(span, count)
        keep.append((d_l, d_r, o, d_p, refiner, count))
        batches.append((i, d_l.data_ptr(), W, Hh, W, W * Hh, d_r.data_ptr(), count, so))
        rx1 = lz.Receiver(n, subch, span, max_frames=1)
        ref1 = lz.Refiner(span, 1)
        d_r1 = torch.empty_like(d_p)
        o1 = [lz.rx_outputs(fmt, 1) for _ in range(count)]
        singles.append((rx1, ref1, d_l, d_p, d_r1, o1))
    streams = sum(f[3] for f in formats)

    # each format's registration on its own stream, forked from the tick's stream and joined back before the engine
    # (the formats' frames are independent; the engine overlaps their receivers the same way)
    sides = [torch.cuda.Stream() for _ in keep]
    fork, joins = torch.cuda.Event(), [torch.cuda.Event() for _ in keep]

    def tick():
        fork.record(stream)
        for (d_l, d_r, o, d_p, refiner, count), side, join in zip(keep, sides, joins):
            side.wait_event(fork)
            with torch.cuda.stream(side):
                d_r.copy_(d_p)
            refiner.refine_dev(d_l.data_ptr(), W, Hh, W * Hh, d_r.data_ptr(), count, 3, None, None, side.cuda_stream)
            join.record(side)
            stream.wait_event(join)
        eng.run_dev(batches, sp)

    def tick_pipelined():
        # each format's registration, then at once its decode (the engine on that format's batch alone, a graph a
        # format), on the format's own stream: a format's decode overlaps the other formats' registrations
        fork.record(stream)
        for (d_l, d_r, o, d_p, refiner, count), side, join, b in zip(keep, sides, joins, batches):
            side.wait_event(fork)
            with torch.cuda.stream(side):
                d_r.copy_(d_p)
            refiner.refine_dev(d_l.data_ptr(), W, Hh, W * Hh, d_r.data_ptr(), count, 3, None, None, side.cuda_stream)
            eng.run_dev([b], side.cuda_stream)
            join.record(side)
            stream.wait_event(join)

    def tick_single():
        for rx1, ref1, d_l, d_p, d_r1, o1 in singles:
            d_r1.copy_(d_p)
            for k, (o, so) in enumerate(o1):
                ref1.refine_dev(d_l[k].data_ptr(), W, Hh, W * Hh, d_r1[k].data_ptr(), 1, 3, None, None, sp)
                lz._check(lz.lib().lizg_rx_finish_luma_dev(rx1._h, lz.ctypes.c_void_p(d_l[k].data_ptr()), W, Hh, W, W * Hh,
                                                           lz.ctypes.c_void_p(d_r1[k].data_ptr()), 1, lz.ctypes.byref(so), None, None,
                                                           lz.ctypes.c_void_p(sp)), "finish_luma")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn, K):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(K):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / K
    def registration():
        fork.record(stream)
        for (d_l, d_r, o, d_p, refiner, count), side, join in zip(keep, sides, joins):
            side.wait_event(fork)
            with torch.cuda.stream(side):
                d_r.copy_(d_p)
            refiner.refine_dev(d_l.data_ptr(), W, Hh, W * Hh, d_r.data_ptr(), count, 3, None, None, side.cuda_stream)
            join.record(side)
            stream.wait_event(join)

    def oks():
        return [o["ok"].cpu().numpy().copy() for _, _, o, _, _, _ in keep]
    K = max(5, args.steps // 3)
    # the engine both ways on the tick's registered frames: a graph a format on its own stream, and stage-wise across
    # the formats (one column pass, row pass and decode grid over every format's items); the tuner keeps the faster
    tick()
    torch.cuda.synchronize()
    ms_reg = timed(registration, K)
    ms_eng, ms_tick, ok_mode = {}, {}, {}
    for mode in (0, 1):
        eng.set_mixed(mode)
        ms_eng[mode] = timed(lambda: eng.run_dev(batches, sp), K)
        ms_tick[mode] = timed(tick, K)
        ok_mode[mode] = (oks(), eng.launches)
    eng.set_mixed(0)
    ms_pipe = timed(tick_pipelined, K)
    ok_pipe = oks()
    tuned, _ = eng.autotune(batches, sp)   # each format's decode tuned on its batch, then the engine's mode
    ms_eng_tuned = timed(lambda: eng.run_dev(batches, sp), K)
    tuned_variants = [[eng.rx_variant(i, t) for t in range(eng.formats[i].tiers)] for i in range(len(formats))]
    ms = timed(tick, K)
    arrangement = "registration, then the engine"
    if ms_pipe < ms:
        eng.set_mixed(0)
        ms, arrangement = timed(tick_pipelined, K), "each format's registration then its decode"
    ms1 = timed(tick_single, max(3, K // 2))
    ok = sum(int(o["ok"].sum().item()) for _, _, o, _, _, _ in keep)
    blocks = sum(f[3] * eng.formats[i].blocks for i, f in enumerate(formats))
    same = all(np.array_equal(o["ok"][k].cpu().numpy(), o1[k][0]["ok"][0].cpu().numpy())
               for (_, _, o, _, _, _), (_, _, _, _, _, o1) in zip(keep, singles) for k in range(len(o1)))
    same_modes = all(np.array_equal(a, b) and np.array_equal(a, c) for a, b, c in zip(ok_mode[0][0], ok_mode[1][0], ok_pipe))
    res = {"workload": "32 streams of 3840x2160 luma at nominal 60 fps; formats n/subch/span 384/64/128 x10, 768/320/128 x8, "
                       "1152/720/256 x6, 1536/1024/256 x5, 1536/1024/512 x3; painted by the sender; rotation 15 deg, tilt 20 deg, "
                       "scale 0.8-1.1 x 1700 px, radial k1 U(+-0.05), blur U(0.5, 2.0) px, AWGN 3 DN; registered on the device "
                       "from a finder's corners (3 rounds of anchors and lens model) inside the tick",
           "streams": streams, "frames_per_s": round(streams / (ms / 1e3), 1), "payload_MBps": round(ok * 472 / (ms / 1e3) / 1e6, 2),
           "ms_per_tick": round(ms, 4), "realtime_60fps_streams": round(streams / (ms / 1e3) / 60, 1),
           "blocks_verified": ok, "blocks": blocks, "block_pass_rate": round(ok / blocks, 4), "gpu_launches_per_tick": ok_mode[tuned if arrangement.startswith("registration") else 0][1],
           "one_frame_a_launch": {"frames_per_s": round(streams / (ms1 / 1e3), 1), "ms_per_tick": round(ms1, 4)},
           "batched_vs_one_frame": round(ms1 / ms, 2), "identical_crc_sets": bool(same),
           "engine_mode": ["a graph a format", "stage-wise across formats"][tuned],
           "registration_ms": round(ms_reg, 4),
           "engine_ms": {"a_graph_a_format": round(ms_eng[0], 4), "stage_wise": round(ms_eng[1], 4),
                         "tuned": round(ms_eng_tuned, 4), "tuned_decode_variants_per_format": tuned_variants},
           "tick_ms": {"a_graph_a_format": round(ms_tick[0], 4), "stage_wise": round(ms_tick[1], 4),
                       "each_format_registered_then_decoded": round(ms_pipe, 4)},
           "tick_arrangement": arrangement,
           "engine_launches": {"a_graph_a_format": ok_mode[0][1], "stage_wise": ok_mode[1][1]},
           "arrangements_identical_crc_sets": bool(same_modes)}
    peak, peak_src = peaks()
    res["hbm"] = {"algorithmic_bytes_per_tick": tick_bytes, "GBps": round(tick_bytes / (ms / 1e3) / 1e9, 1),
                  "frac": round(tick_bytes / (ms / 1e3) / 1e9 / peak, 4),
                  "one_frame_a_launch_frac": round(tick_bytes / (ms1 / 1e3) / 1e9 / peak, 4), "peak_GBps": peak, "peak_source": peak_src,
                  "bytes": "luma footprint + Y written and read + used coefficients and soft values written and read + blocks (the "
                           "registration's reads not counted)"}
    for _, _, _, _, refiner, _ in keep:
        refiner.close()
    for _, ref1, _, _, _, _ in singles:
        ref1.close()
    eng.close()
    return res


def bench_ingest(args, stream):
    """Camera-format ingest to luma on the GPU, 16 frames a call of smooth synthetic scenes with sensor noise: 3840 x 2160
    RGBA8 (liz_decode's conversion), and a 3840 x 2160 sensor's RAW10 developed at bin 1 (3840 x 2160 out) and bin 2
    (1920 x 1080 out), and P010. Device-timed;
    GB/s = the frames' bytes read (the whole plane a format's samples occupy) and written over the time; the fraction is
    of the measured HBM copy peak. Beside it the same conversions on the host cores (the oracle's C, a frame a thread)."""
    import concurrent.futures
    import numpy as np
    import torch
    import lizard_gb300 as lz
    import oracle
    frames, W, H = 16, 3840, 2160
    peak, peak_src = peaks()
    rng = np.random.default_rng(77)
    # smooth scenes, as a camera sees them: gradients and a ripple, sensor noise, 10 bits
    yy, xx = np.mgrid[0:H, 0:W].astype(np.float32)

    def scene(k):
        v = 120 + 700 * xx / W + 90 * np.sin(yy / (40.0 + k) + k) + rng.normal(0, 6, (H, W)).astype(np.float32)
        return np.clip(np.rint(v), 0, 1023).astype(np.uint16)

    def pack(kind, v):
        if kind is None:   # RGBA8: the scene in three tinted channels
            g = (v >> 2).astype(np.uint8)
            return np.stack([g, (g * 0.9).astype(np.uint8), (g * 0.8).astype(np.uint8), np.full_like(g, 255)], -1).reshape(H, -1)
        if kind == 0:      # P010: ten bits at the top of little-endian 16-bit samples
            w16 = (v.astype(np.uint16) << 6)
            return np.stack([(w16 & 255).astype(np.uint8), (w16 >> 8).astype(np.uint8)], -1).reshape(H, -1)
        g4 = v.reshape(H, W // 4, 4)   # RAW10: four samples' top bytes, then their low bits
        low = (g4[..., 0] & 3) | ((g4[..., 1] & 3) << 2) | ((g4[..., 2] & 3) << 4) | ((g4[..., 3] & 3) << 6)
        return np.concatenate([(g4 >> 2).astype(np.uint8), low[..., None].astype(np.uint8)], -1).reshape(H, -1)
    scenes = [scene(k) for k in range(4)]
    sp = stream.cuda_stream
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    lv = (lz.ctypes.c_float * 9)(64.0, 66.0, 63.0, 65.0, 1023.0, 1.9, 1.0, 1.0, 1.6)
    res = {}
    cases = [("rgba8_3840x2160", 4 * W, H, W, H, None), ("raw10_bin1_3840x2160", (W + 3) // 4 * 5, H, W, H, 1),
             ("raw10_bin2_to_1920x1080", (W + 3) // 4 * 5, H, W // 2, H // 2, 2), ("p010_3840x2160", 2 * W, H, W, H, 0)]
    if not os.path.exists(oracle.PORT_PATH):
        oracle.build(ref=False)
    for name, rowb, rows, w, h, kind in cases:
        host = np.stack([pack(kind, scenes[f % 4]).reshape(-1) for f in range(frames)])
        assert host.shape[1] == rows * rowb
        d_in = torch.from_numpy(host).cuda()
        d_out = torch.zeros((frames, h, w), dtype=torch.uint8, device="cuda")
        if kind is None:
            def call():
                lz._check(lz.lib().lizg_ingest_pixels_dev(lz.ctypes.c_void_p(d_in.data_ptr()), W, H, rowb, rows * rowb, 3, frames,
                                                          lz.ctypes.c_void_p(d_out.data_ptr()), lz.ctypes.c_void_p(sp)), "ingest")
        else:
            fmt = 0x36 if kind == 0 else 0x25
            r = lz.RawFrame(fmt, rowb, 2, 0, 0, max(kind, 1), lv)

            def call():
                lz._check(lz.lib().lizg_develop_dev(lz.ctypes.byref(r), lz.ctypes.c_void_p(d_in.data_ptr()), rows * rowb, rows * rowb, frames,
                                                    0, 0, w, h, lz.ctypes.c_void_p(d_out.data_ptr()), lz.ctypes.c_void_p(sp)), "develop")
        for _ in range(3):
            call()
        torch.cuda.synchronize()
        reps = 20
        e0.record(stream)
        for _ in range(reps):
            call()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        moved = frames * (rows * rowb + w * h)
        gbs = moved / (ms / 1e3) / 1e9
        # the host cores: the same conversion of every frame once

        def cpu(f):
            o = np.zeros((h, w), np.uint8)
            if kind is None:
                oracle.port().orc_ingest_pixels(oracle._p(host[f]), W, H, rowb, 3, oracle._p(o))
            else:
                oracle.port().orc_develop(0x36 if kind == 0 else 0x25, oracle._p(host[f]), rowb, 2, 0, 0, max(kind, 1),
                                          oracle._p(np.array(list(lv), np.float32)), 0, 0, w, h, oracle._p(o), w)
            return o
        t0 = time.perf_counter()
        with concurrent.futures.ThreadPoolExecutor(os.cpu_count() or 1) as ex:
            outs = list(ex.map(cpu, range(frames)))
        dt = time.perf_counter() - t0
        same = all(np.array_equal(outs[f], d_out[f].cpu().numpy()) for f in (0, frames - 1))
        res[name] = {"frames_per_s": round(frames / (ms / 1e3), 1), "GBps": round(gbs, 1), "hbm_frac": round(gbs / peak, 4),
                     "ms_per_call": round(ms, 4), "identical_to_host": bool(same),
                     "cpu": {"frames_per_s": round(frames / dt, 1), "cores": os.cpu_count() or 1, "kind": "port"}}
    res["peak"] = {"GBps": peak, "source": peak_src}
    return res


def bench_border_nodes(args, stream):
    """The registration's border nodes (lizg_border_nodes_dev): refine_node over the border lattice of 64 distinct captured
    1920 x 1080 frames, each LIZARD-1024 (n = 1536) in the 128 ring at about 2.6 pixels a module, rotated
    up to 15 degrees, H put up to a pixel off. Device-timed with CUDA events; every distinct frame's nodes checked
    identical to the oracle's (the reference's portable build, restated); beside it the oracle on the host cores, a
    frame a thread."""
    import concurrent.futures
    import numpy as np
    import torch
    import lizard_gb300 as lz
    from lizard_gb300_testing import synth
    import oracle
    span, n, subch, W, Hh, frames = 256, 1536, 1024, 1920, 1080, 64
    nn = synth.layout_nodes(span).size
    d_l, Hws = warped_frames(n, subch, span, W, Hh, frames, 800, (0.42, 0.45))
    lumas = list(d_l.cpu().numpy())
    Hs = []
    for k in range(frames):
        rng = np.random.default_rng(10800 + k)
        H = (Hws[k] / Hws[k][2, 2]).astype(np.float32).ravel()
        H[2] += np.float32(rng.uniform(-1, 1))
        H[5] += np.float32(rng.uniform(-1, 1))
        Hs.append(H)
    d_h = torch.from_numpy(np.stack(Hs)).cuda()
    d_n = torch.zeros((frames, nn, nn, 4), dtype=torch.float32, device="cuda")
    sp = stream.cuda_stream

    def call():
        lz._check(lz.lib().lizg_border_nodes_dev(span, lz.ctypes.c_void_p(d_l.data_ptr()), W, Hh, W * Hh, lz.ctypes.c_void_p(d_h.data_ptr()), 9,
                                                 None, frames, lz.ctypes.c_void_p(d_n.data_ptr()), lz.ctypes.c_void_p(sp)), "border_nodes")
    for _ in range(3):
        call()
    torch.cuda.synchronize()
    reps = max(5, args.steps // 3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        call()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    got = d_n.cpu().numpy()
    P = oracle.port()

    def host(k):
        out = np.zeros(4 * nn * nn, np.float32)
        P.orc_border_nodes(span, oracle._p(lumas[k]), W, Hh, oracle._p(Hs[k]), None, oracle._p(out))
        return out.reshape(nn, nn, 4)
    same = all(np.array_equal(got[k].view(np.uint32), host(k).view(np.uint32)) for k in range(frames))
    marked = 4 * (nn - 2)
    held = int((got[..., 2] >= 0.35).sum())
    threads = os.cpu_count() or 1
    done, t0 = 0, time.perf_counter()
    with concurrent.futures.ThreadPoolExecutor(threads) as ex:
        while time.perf_counter() - t0 < 2.0:
            list(ex.map(host, range(frames)))
            done += frames
    dt = time.perf_counter() - t0
    return {"workload": "border nodes (refine_node over the 128 ring's border lattice, %d nodes a frame), 64 distinct frames of 1920x1080, LIZARD-1024 "
                        "painted by the sender at ~2.6 px a module, rotation up to 15 deg, H up to a pixel off, AWGN 3 DN" % marked,
            "frames_per_s": round(frames / (ms / 1e3), 1), "nodes_per_s": round(frames * marked / (ms / 1e3), 1), "ms_per_call": round(ms, 4),
            "nodes_held": held, "nodes": frames * marked, "gpu_launches_per_call": 1, "identical_to_oracle": bool(same),
            "cpu": {"frames_per_s": round(done / dt, 1), "cores": threads, "kind": "port",
                    "sample": "the 64 frames repeatedly for %.1f s, a frame a thread" % dt}}


def bench_fmt_word(args, stream):
    """The format word (lizg_fmt_read_dev): its read off the border of a batch of 2048 registered 1280 x 720 frames
    (the 128 ring's word, RS(32, 3); 32 distinct captures at about 2 pixels a module, rotation up to 12 degrees, blur
    0.5-1.5 pixels, AWGN, a quarter with glare over a side so that the decode needs erasures) and its decode, one
    launch. Device-timed with CUDA events; the soft values and words checked identical to the oracle's on every
    distinct capture; beside it the oracle's read and decode on the host cores, a frame a thread."""
    import concurrent.futures
    import numpy as np
    import torch
    import lizard_gb300 as lz
    from lizard_gb300_testing import synth
    import oracle
    span, W, Hh, frames, distinct = 256, 1280, 720, 2048, 32
    lumas, regs, words = [], [], []
    for k in range(distinct):
        rng = np.random.default_rng(900 + k)
        version, fps = int(rng.integers(4, 65)), int(rng.integers(0, 256))
        glare = None
        if k % 4 == 3:
            glare = (float(rng.choice([W / 2, W - 200, 200])), float(rng.choice([60, Hh - 60, Hh / 2])), 150.0, 3.0)
        luma, reg, _ = synth.word_capture(span, 2, version, fps, W, Hh, rng, blur=float(rng.uniform(0.5, 1.5)), sigma=3.0, glare=glare)
        lumas.append(luma)
        regs.append(reg)
        words.append((version, fps))
    cells, _ = synth.fmt_geometry(span)
    d_l = torch.from_numpy(np.stack([lumas[k % distinct] for k in range(frames)])).cuda()
    d_r = torch.from_numpy(np.stack([regs[k % distinct] for k in range(frames)])).cuda()
    d_q = torch.zeros((frames, 4 * cells), dtype=torch.float32, device="cuda")
    d_w = torch.zeros((frames, 4), dtype=torch.int32, device="cuda")
    sp = stream.cuda_stream

    def call():
        lz._check(lz.lib().lizg_fmt_read_dev(span, lz.ctypes.c_void_p(d_l.data_ptr()), W, Hh, W * Hh, lz.ctypes.c_void_p(d_r.data_ptr()), d_r.shape[1],
                                             frames, lz.ctypes.c_void_p(d_q.data_ptr()), lz.ctypes.c_void_p(d_w.data_ptr()), lz.ctypes.c_void_p(sp)), "fmt_read")
    for _ in range(3):
        call()
    torch.cuda.synchronize()
    reps = max(5, args.steps // 3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        call()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    word, q = d_w.cpu().numpy(), d_q.cpu().numpy()
    if not os.path.exists(oracle.PORT_PATH):
        oracle.build(ref=False)
    nodes = synth.layout_nodes(span).astype(np.float32)
    P = oracle.port()
    _, nbytes = synth.fmt_geometry(span)

    def host(k):
        qo = np.zeros(4 * cells, np.float32)
        got = P.orc_fmt_read(span, oracle._p(lumas[k]), W, Hh, oracle._p(regs[k]), oracle._p(nodes), nodes.size, oracle._p(qo))
        vf = np.zeros(2, np.int32)
        ok = bool(got) and P.orc_fmt_decode(oracle._p(qo), cells, nbytes, oracle._p(vf)) == 0
        return qo, [int(got > 0), int(ok), int(vf[0]) if ok else 0, int(vf[1]) if ok else 0]
    same = True
    for k in range(distinct):
        qo, wo = host(k)
        same &= list(word[k]) == wo and (not wo[0] or np.array_equal(q[k].view(np.uint32), qo.view(np.uint32)))
    threads = os.cpu_count() or 1
    done, t0 = 0, time.perf_counter()
    with concurrent.futures.ThreadPoolExecutor(threads) as ex:
        while time.perf_counter() - t0 < 2.0:
            list(ex.map(host, range(distinct)))
            done += distinct
    dt = time.perf_counter() - t0
    right = sum(int(word[k][1] == 1 and (word[k][2], word[k][3]) == words[k % distinct]) for k in range(frames))
    return {"workload": "format word read + RS(32,3) soft decode, 2048 registered 1280x720 frames, 128 ring at ~2 px a module, blur 0.5-1.5 px, AWGN 3 DN, a quarter with glare over a side",
            "frames_per_s": round(frames / (ms / 1e3), 1), "ms_per_call": round(ms, 4), "words_right": right, "frames": frames,
            "gpu_launches_per_call": 1, "identical_to_oracle": bool(same),
            "cpu": {"frames_per_s": round(done / dt, 1), "cores": threads, "kind": "port",
                    "sample": "the 32 distinct frames read and decoded repeatedly for %.1f s, a frame a thread" % dt}}


def bench_encoder(args, stream):
    """The sender on the GPU (lizg_encode_dev): seeded blocks to the ring's grey page, a batch a call: LIZARD-1024
    (n = 1536) in the 128 ring (1740 x 1740 pages, 6 pixels a module) and LIZARD-64 (n = 384) in the 64 ring (486 x 486).
    Device-timed with CUDA events; the first page of each checked against the oracle (the numpy restatement of the
    reference's lizard_encode, grey levels within one at rounding ties); beside it the oracle on one host core."""
    import numpy as np
    import torch
    import lizard_gb300 as lz
    from lizard_gb300_testing import synth
    res = {}
    for name, (n, subch, span, frames) in (("lizard1024_128ring", (1536, 1024, 256, 32)), ("lizard64_64ring", (384, 64, 128, 256))):
        fmt = lz.Format(n, subch, span)
        enc = lz.Encoder(n, subch, span, max_frames=frames)
        blocks = np.stack([synth.random_blocks(fmt.blocks, 700 + k) for k in range(frames)])
        d_b = torch.from_numpy(blocks).cuda()
        d_g = torch.zeros((frames, enc.W, enc.W), dtype=torch.uint8, device="cuda")
        sp = stream.cuda_stream

        def call():
            lz._check(lz.lib().lizg_encode_dev(enc._h, lz.ctypes.c_void_p(d_b.data_ptr()), frames, 1, None, lz.ctypes.c_void_p(d_g.data_ptr()),
                                               lz.ctypes.c_void_p(sp)), "encode")
        for _ in range(3):
            call()
        torch.cuda.synchronize()
        reps = max(5, args.steps // 3)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            call()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        t0 = time.perf_counter()
        _, g = synth.encode_drive(fmt, blocks[0], parity=1)
        dt = time.perf_counter() - t0
        diff = d_g[0].cpu().numpy().astype(int) - g.astype(int)
        res[name] = {"frames_per_s": round(frames / (ms / 1e3), 1), "ms_per_call": round(ms, 4), "frames": frames, "page": [enc.W, enc.W],
                     "page_GBps": round(frames * enc.W * enc.W / (ms / 1e3) / 1e9, 2), "blocks_per_frame": fmt.blocks,
                     "within_one_of_oracle": bool(np.abs(diff).max() <= 1), "grey_off_by_one": int(np.count_nonzero(diff)),
                     "gpu_launches_per_call": 6, "cpu": {"frames_per_s": round(1 / dt, 2), "cores": 1, "kind": "port",
                                                          "sample": "one page by the numpy oracle (FP64 transform), one core"}}
    return res


def bench_refinement(args, stream):
    """The full receiver on distorted captures (the distorted full receiver's configuration): 1920 x 1080 frames, one
    LIZARD-1024 (n = 1536) symbol in the 128 ring painted by the sender (the library's GPU encoder: the reference's
    page with its border and the picture's cyclic guard), seen through rotation U(+-15 deg), tilt U(+-20 deg) about a
    random in-plane axis, the layout's side 1000 px x U(0.8, 1.1), radial k1 about the frame centre, Gaussian blur in
    linear light (gamma 2.2), AWGN 3 DN, a seed a frame (lizard_gb300_testing.render, on the GPU). Registrations:
    corners = the homography through the layout's four corners as the camera sees them (a finder's), no lens; plain
    (the configuration's: homography + anchors) = + three rounds of the anchor search and the lens model the anchors
    give, written into the node mesh (lizg_refine_dev); anchor_register = the reference's whole registration from the
    anchors (lizg_anchor_register_dev: up to six rounds, H refitted from the anchors each round, the robust model, the
    corners judged and searched again, H made again, the model about H); refined = the plain registration's decode, then the frames it
    left blocks unverified in refined by three Gauss-Newton steps of the adjoint refinement (H and the 7 x 7 anchor
    field against the pilots, the timing track and the anchors' centres, lizg_field_refine_dev) and decoded again;
    bound = the camera's true map at every node (no registration can do better). Three sets:
    the configuration's 1024 frames (k1 U(+-0.05), blur U(0.5, 2.0)), blur 1.5 px / k1 0.03, blur 0.5 px / k1 U(+-0.05).
    Device-timed."""
    import numpy as np
    import torch
    import lizard_gb300 as lz
    from lizard_gb300_testing import render, synth
    n, subch, span, W, Hh = 1536, 1024, 256, 1920, 1080
    fmt = lz.Format(n, subch, span)
    rng = np.random.default_rng(123)
    sets = [("spread", [(9000 + k, float(rng.uniform(-0.05, 0.05)), float(rng.uniform(0.5, 2.0))) for k in range(1024)]),
            ("blur1.5_k1_0.03", [(9100 + k, 0.03, 1.5) for k in range(64)]),
            ("mild_blur0.5", [(9200 + k, float(rng.uniform(-0.05, 0.05)), 0.5) for k in range(64)])]
    if getattr(args, "refine_frames", 0):
        sets = [("spread", sets[0][1][:args.refine_frames])]
    sp = stream.cuda_stream
    res = {"workload": "1920x1080, LIZARD-1024 (n=1536) in the 128 ring painted by the sender (border, cyclic guard), rotation 15 deg, "
                       "tilt 20 deg, scale 0.8-1.1 x 1000 px, radial k1, blur in linear light, AWGN 3 DN, a seed a frame; corners = a finder's "
                       "homography; plain = + 3 rounds of anchors and lens model (homography + anchors); refined = + 3 Gauss-Newton steps "
                       "against the pilots; bound = the true map at every node"}
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    rx = lz.Receiver(n, subch, span, max_frames=1024)
    ref = lz.Refiner(span, 1024)
    fld = lz.FieldRefiner(n, subch, span, chunk=152)   # a frame an SM for the step's solve
    for name, js in sets:
        frames = len(js)
        seeds = [j[0] for j in js]
        vs = render.views(n, span, W, Hh, seeds, 1000.0)
        blocks = np.stack([synth.random_blocks(fmt.blocks, s) for s in seeds])
        pg, pxm = render.pages(lz, n, subch, span, blocks, 1)
        d_l = torch.empty((frames, Hh, W), dtype=torch.uint8, device="cuda")
        for k, (s, k1, blur) in enumerate(js):
            d_l[k] = render.capture(pg[k], pxm, W, Hh, vs[k], k1, blur, 3.0, s)
        del pg
        d_plain = torch.from_numpy(np.stack([render.registration(span, vs[k], js[k][1], W, Hh) for k in range(frames)])).cuda()
        d_true = torch.from_numpy(np.stack([render.registration(span, vs[k], js[k][1], W, Hh, true_mesh=True) for k in range(frames)])).cuda()
        stride = d_plain.shape[1]
        d_a = torch.empty_like(d_plain)
        d_g = torch.empty_like(d_plain)
        d_found = torch.zeros(frames, dtype=torch.int32, device="cuda")
        d_lens = torch.zeros((frames, 15), dtype=torch.float64, device="cuda")
        d_gate = torch.zeros(frames, dtype=torch.uint8, device="cuda")
        d_imp = torch.zeros(frames, dtype=torch.int32, device="cuda")
        ao = {"ok": torch.zeros((frames, 49), dtype=torch.uint8, device="cuda")}
        for key in ("peak", "dx", "dy", "u", "v"):
            ao[key] = torch.zeros((frames, 49), dtype=torch.float32, device="cuda")
        a_out = lz.AnchorOut(*[ao[key].data_ptr() for key in ("ok", "peak", "dx", "dy", "u", "v")])
        outs = {t: rx._outputs(frames, torch, keep=False) for t in ("corners", "plain", "anchor_register", "first", "refined", "bound")}
        d_ar = torch.empty_like(d_plain)
        d_union = torch.zeros((frames, fmt.blocks), dtype=torch.uint8, device="cuda")

        def finish(d_reg, tag):
            lz._check(lz.lib().lizg_rx_finish_luma_dev(rx._h, lz.ctypes.c_void_p(d_l.data_ptr()), W, Hh, W, W * Hh, lz.ctypes.c_void_p(d_reg.data_ptr()),
                                                       frames, lz.ctypes.byref(outs[tag][1]), None, None, lz.ctypes.c_void_p(sp)), "finish_luma")

        def anchors(d_reg):
            d_reg.copy_(d_plain)
            ref.refine_dev(d_l.data_ptr(), W, Hh, W * Hh, d_reg.data_ptr(), frames, 3, d_found.data_ptr(), d_lens.data_ptr(), sp)

        def registered():
            # the reference's own registration from the anchors (anchor_register: H refitted each round, the robust
            # model, the corners judged and searched again, H made again), then the decode
            d_ar.copy_(d_plain)
            ref.register_dev(d_l.data_ptr(), W, Hh, W * Hh, d_ar.data_ptr(), frames, stream=sp)
            finish(d_ar, "anchor_register")

        def refined():
            # the plain registration and decode; then the frames it left blocks unverified in, refined by the adjoint
            # (H and the anchor field against the pilots, the track and the anchors' centres) and decoded again; a
            # block verified by either decode is the frame's (the CRC-32C decides, as a receiver keeps any block it
            # verifies)
            anchors(d_g)
            finish(d_g, "first")
            d_gate.copy_((outs["first"][0]["ok"].sum(dim=1) < fmt.blocks).to(torch.uint8))
            lz._check(lz.lib().lizg_anchor_find_dev(span, lz.ctypes.c_void_p(d_l.data_ptr()), W, Hh, W * Hh, lz.ctypes.c_void_p(d_g.data_ptr()), stride,
                                                    lz.ctypes.c_void_p(d_lens.data_ptr()), None, frames, lz.ctypes.byref(a_out), lz.ctypes.c_void_p(sp)),
                      "anchor_find")
            fld.refine_dev(d_l.data_ptr(), W, Hh, W * Hh, d_g.data_ptr(), frames, 3, a_out, d_gate.data_ptr(), None, d_imp.data_ptr(), sp)
            finish(d_g, "refined")
            torch.maximum(outs["refined"][0]["ok"], outs["first"][0]["ok"], out=d_union)

        paths = {"corners": lambda: finish(d_plain, "corners"),
                 "plain": lambda: (anchors(d_a), finish(d_a, "plain")),
                 "anchor_register": registered,
                 "refined": refined,
                 "bound": lambda: finish(d_true, "bound")}
        out = {"frames": frames}
        for tag, fn in paths.items():
            fn()
            torch.cuda.synchronize()
            reps = 2 if tag == "refined" else 3
            e0.record(stream)
            for _ in range(reps):
                fn()
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / reps
            def rates(ok):
                return {"blocks_verified": int(ok.sum()), "blocks": int(ok.size), "block_pass_rate": round(float(ok.mean()), 4),
                        "frames_with_a_block": int((ok.sum(axis=1) > 0).sum()), "frames_all_blocks": int(ok.all(axis=1).sum()),
                        "frames_per_s": round(frames / (ms / 1e3), 1)}
            out[tag] = rates((d_union if tag == "refined" else outs[tag][0]["ok"]).cpu().numpy())
            if tag == "refined":
                out["refined_registration_alone"] = rates(outs["refined"][0]["ok"].cpu().numpy())
        out["anchors_found_mean"] = round(float(d_found.float().mean().item()), 1)
        out["refined_frames"] = int(d_gate.sum().item())
        out["refined_steps_kept_frames"] = int(d_imp.sum().item())
        out["plain_points_over_corners"] = round(100 * (out["plain"]["block_pass_rate"] - out["corners"]["block_pass_rate"]), 2)
        out["refined_points_over_plain"] = round(100 * (out["refined"]["block_pass_rate"] - out["plain"]["block_pass_rate"]), 2)
        out["bound_points_over_plain"] = round(100 * (out["bound"]["block_pass_rate"] - out["plain"]["block_pass_rate"]), 2)
        out["anchor_register_points_over_plain"] = round(100 * (out["anchor_register"]["block_pass_rate"] - out["plain"]["block_pass_rate"]), 2)
        res[name] = out
        del d_l
    ref.close()
    fld.close()
    return res


def run_reference(args, rank, ws):
    """The reference arm: the reference's CPU decoder on the host cores, same metric and workload."""
    if rank != 0:
        return
    from lizard_gb300_testing import synth
    import oracle
    if not os.path.exists(oracle.PORT_PATH):
        oracle.build(ref=False)
    batch = synth.ldpc_batch(args.count, seed=1000)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_decode(batch, threads, min(args.count, 4096))
    vals, secs = [], []
    kind = None
    for _ in range(args.steps):
        v, dt, kind = cpu_decode(batch, threads, args.count)
        vals.append(v); secs.append(dt)
    value = args.count * 3840 * len(secs) / sum(secs) / 1e9
    print(json.dumps({"impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": args.gpus,
                      "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * sum(secs) / len(secs), 3),
                      "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int8/int16",
                      "data": "synthetic", "config": workload(args.count),
                      "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": threads, "kind": kind,
                                       "sample": "the whole %d-codeword batch a step" % args.count,
                                       "reference_estimate": reference_estimate(value, kind)},
                      "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))


def bench_noalloc(batch, d_llr, stream):
    """The allocation-free decode (lizg_ldpc_decode_noalloc: the four codes one after another on the caller's stream)
    against a plan (the codes overlapped on side streams) on the batch's first LIZG_NOALLOC_MAX_CODEWORDS codewords,
    device-resident; outputs checked identical."""
    import ctypes
    import numpy as np
    import torch
    import lizard_gb300 as lz
    count = 8192
    rates = np.ascontiguousarray(batch["rates"][:count])
    plan = lz.LdpcPlan(rates, MAX_ITER, STALL_IT, STALL_RATIO)
    fn = lz.lib().lizg_ldpc_decode_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float] + [ctypes.c_void_p] * 4
    d_rate = torch.from_numpy(rates).cuda()
    outs = [(torch.empty(plan.llr_bytes // 8, dtype=torch.uint8, device="cuda"), torch.empty(count, dtype=torch.int32, device="cuda"),
             torch.empty(count, dtype=torch.uint8, device="cuda")) for _ in range(2)]
    sp = stream.cuda_stream
    calls = {"plan": lambda o: plan.run_dev(d_llr.data_ptr(), o[0].data_ptr(), o[1].data_ptr(), o[2].data_ptr(), sp),
             "noalloc": lambda o: lz._check(fn(d_llr.data_ptr(), d_rate.data_ptr(), count, MAX_ITER, STALL_IT, STALL_RATIO, o[0].data_ptr(),
                                                  o[1].data_ptr(), o[2].data_ptr(), sp), "lizg_ldpc_decode_noalloc")}
    res = {"workload": "the first %d codewords of the batch, device-resident" % count}
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for (name, call), o in zip(calls.items(), outs):
        for _ in range(3):
            call(o)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(20):
            call(o)
        e1.record(stream)
        torch.cuda.synchronize()
        res[name + "_ms"] = round(e0.elapsed_time(e1) / 20, 4)
    res["identical"] = all(torch.equal(a, b) for a, b in zip(outs[0], outs[1]))
    res["noalloc_over_plan_time"] = round(res["noalloc_ms"] / res["plan_ms"], 3)
    return res


def bench_ldpc_variants(args, stream):
    """Each code's codewords of the workload batch decoded by every kernel variant of that code: ms a decode of them,
    and whether bits and iteration counts equal variant 0's. Launch order: code by code (7/8, 3/4, 2/3, 1/2), variant
    by variant, 2 untimed then 5 timed launches each."""
    import numpy as np
    import torch
    import lizard_gb300 as lz
    from lizard_gb300_testing import synth
    b = synth.ldpc_batch(args.count, seed=1000)
    out = {}
    for name, r in zip(("7/8", "3/4", "2/3", "1/2"), (6, 4, 3, 2)):
        sel = np.nonzero(b["rates"] == r)[0]
        n = lz.CODE_N[r]
        llr = np.concatenate([b["llr"][b["offsets"][i]:b["offsets"][i] + n] for i in sel])
        plan = lz.LdpcPlan(np.full(sel.size, r, np.int32), MAX_ITER, STALL_IT, STALL_RATIO)
        d_llr = torch.from_numpy(llr).cuda()
        d_bits = torch.empty(plan.llr_bytes // 8, dtype=torch.uint8, device="cuda")
        d_its = torch.empty(plan.count, dtype=torch.int32, device="cuda")
        d_ok = torch.empty(plan.count, dtype=torch.uint8, device="cuda")
        run = lambda: plan.run_dev(d_llr.data_ptr(), d_bits.data_ptr(), d_its.data_ptr(), d_ok.data_ptr(), stream.cuda_stream)
        first, rows = None, []
        for v in range(lz.ldpc_variants(r)):
            lz.ldpc_set_variant(r, v)
            for _ in range(2):
                run()
            torch.cuda.synchronize()
            got = (d_bits.cpu().numpy(), d_its.cpu().numpy())
            first = first or got
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(5):
                run()
            e1.record(stream)
            torch.cuda.synchronize()
            _, wpc, loop, pair = lz.ldpc_variant(r)
            rows.append({"index": v, "warps_a_codeword": wpc, "loop_form": loop, "pair_form": pair,
                         "ms": round(e0.elapsed_time(e1) / 5, 3),
                         "identical": bool(np.array_equal(got[0], first[0]) and np.array_equal(got[1], first[1]))})
        lz.ldpc_set_variant(r, 0)
        out[name] = {"codewords": int(sel.size), "variants": rows}
    return out


def main():
    args = parse()
    rank, ws, local = dist_init()
    if args.impl == "reference":
        run_reference(args, rank, ws)
        return
    import numpy as np
    import torch
    import lizard_gb300 as lz
    from lizard_gb300_testing import synth
    assert torch.cuda.is_available(), "bench.py needs a CUDA device"
    dev = local
    torch.cuda.set_device(dev)
    if args.ingest_only:
        print(json.dumps({"ingest": bench_ingest(args, torch.cuda.current_stream())}))
        return
    if args.fmt_only:
        print(json.dumps({"format_word": bench_fmt_word(args, torch.cuda.current_stream()),
                          "border_nodes": bench_border_nodes(args, torch.cuda.current_stream())}))
        return
    if args.refine_only:
        print(json.dumps({"refinement": bench_refinement(args, torch.cuda.current_stream())}))
        return
    if args.encode_only:
        print(json.dumps({"sender": bench_encoder(args, torch.cuda.current_stream())}))
        return
    if args.ldpc_variants:
        print(json.dumps({"ldpc_variants": bench_ldpc_variants(args, torch.cuda.current_stream())}))
        return
    tune = None
    if not args.no_autotune:
        # the decoder's kernel variant per code chosen by timing on this device, before any timed work
        t_tune = time.perf_counter()
        chosen = lz.ldpc_autotune(8192, synth.EBN0_SWEEP_DB)
        tune = {"variant": {name: {"index": v, "warps_a_codeword": lz.ldpc_variant(r)[1], "loop_form": lz.ldpc_variant(r)[2], "pair_form": lz.ldpc_variant(r)[3]}
                            for name, r, v in zip(("7/8", "3/4", "2/3", "1/2"), (6, 4, 3, 2), chosen)},
                "seconds": round(time.perf_counter() - t_tune, 2), "calibration": "8192 codewords a code, all-zero codeword, BPSK/AWGN over the workload's Eb/N0 sweep"}
    if args.multistream_only:
        print(json.dumps({"receiver": {"multistream": bench_multistream(args, torch.cuda.current_stream())}}))
        return
    if args.receiver_only:
        st = torch.cuda.current_stream()
        rec = bench_receiver(args, st)
        rec["multistream"] = bench_multistream(args, st)
        print(json.dumps({"receiver": rec, "registration": {"anchor_search": bench_anchor(args, st), "refinement": bench_refinement(args, st),
                                                            "format_word": bench_fmt_word(args, st), "border_nodes": bench_border_nodes(args, st)},
                          "sender": bench_encoder(args, st),
                          "ingest": bench_ingest(args, st)}))
        return
    batch = synth.ldpc_batch(args.count, seed=1000 + rank)
    plan = lz.LdpcPlan(batch["rates"], MAX_ITER, STALL_IT, STALL_RATIO)
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    d_llr = torch.from_numpy(batch["llr"]).to("cuda")
    d_bits = torch.empty(plan.llr_bytes // 8, dtype=torch.uint8, device="cuda")
    d_its = torch.empty(plan.count, dtype=torch.int32, device="cuda")
    d_ok = torch.empty(plan.count, dtype=torch.uint8, device="cuda")

    def step():
        plan.run_dev(d_llr.data_ptr(), d_bits.data_ptr(), d_its.data_ptr(), d_ok.data_ptr(), sp)

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    its = d_its.cpu().numpy()
    ok = d_ok.cpu().numpy()
    bits_dev = d_bits.cpu().numpy()
    edges = lz.edge_updates(its, batch["rates"], MAX_ITER, STALL_IT)

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(dev) as clk:
        barrier(ws)
        torch.cuda.synchronize()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for i in range(args.steps):
            ev[i][0].record(stream)
            step()
            ev[i][1].record(stream)
        t1.record(stream)
        torch.cuda.synchronize()
        barrier(ws)
    elapsed_ms = max_over_ranks(t0.elapsed_time(t1), ws)
    launch_ms = statistics.mean(a.elapsed_time(b) for a, b in ev)
    launches = plan.launches * args.steps
    ms = elapsed_ms / args.steps
    value = ws * args.count * 3840 / (ms / 1e3) / 1e9

    e2e = None
    if not args.no_e2e:
        h_llr = torch.from_numpy(batch["llr"]).pin_memory()
        h_bits = torch.empty(plan.llr_bytes // 8, dtype=torch.uint8).pin_memory()
        h_its = torch.empty(plan.count, dtype=torch.int32).pin_memory()
        h_ok = torch.empty(plan.count, dtype=torch.uint8).pin_memory()
        nb, ni, no = h_llr.numpy(), h_bits.numpy(), h_its.numpy()
        nk = h_ok.numpy()

        def timed_host_runs():
            for _ in range(max(args.warmup, 3)):
                plan.run(nb, ni, no, nk, sp)
            ni.fill(0)   # the timed runs write the outputs checked below
            no.fill(0)
            nk.fill(0)
            barrier(ws)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(args.steps):
                plan.run(nb, ni, no, nk, sp)
            e1.record(stream)
            torch.cuda.synchronize()
            assert np.array_equal(no, its) and np.array_equal(nk, ok) and np.array_equal(ni, bits_dev)
            return max_over_ranks(e0.elapsed_time(e1), ws) / args.steps

        # pinned host buffers: the decoder reads the LLRs and writes its results in host memory (NVLink-C2C)
        e_ms = timed_host_runs()
        in_place = plan.transfer
        # the same buffers staged through device memory: copies in and out on the copy engines, two chunks
        plan.set_transfer(0)
        s_ms = timed_host_runs()
        plan.set_transfer(1)
        gbit = lambda t: round(ws * args.count * 3840 / (t / 1e3) / 1e9, 4)
        e2e = {"value": gbit(e_ms), "unit": UNIT,
               "h2d_bytes_per_step": int(plan.llr_bytes), "d2h_bytes_per_step": int(plan.llr_bytes // 8 + plan.count * 5),
               "ms_per_step": round(e_ms, 3),
               "route": "pinned host buffers read and written in place by the decoder over NVLink-C2C" if in_place
               else "staged through device memory",
               "staged": {"value": gbit(s_ms), "ms_per_step": round(s_ms, 3),
                          "route": "the same pinned buffers copied in and out by cudaMemcpyAsync, two chunks pipelined"}}

    noalloc = bench_noalloc(batch, d_llr, stream) if rank == 0 else None
    if rank != 0:
        return
    alg_bytes = plan.llr_bytes + plan.llr_bytes // 8 + plan.count * 5
    peak, peak_src = peaks()
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    clocks = clk.summary()
    sm_mhz = clocks.get("sm_mhz") if isinstance(clocks, dict) else None
    achieved = alg_bytes / (launch_ms / 1e3) / 1e9
    traffic = traffic_per_step(args.count)
    out = {
        "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": max(args.warmup, 3),
        "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "int8/int16", "data": "synthetic (seeded blocks over a simulated AWGN channel)", "config": workload(args.count),
        "payload_MBps": round(ws * float(ok[its > 0].sum()) * 472 / (ms / 1e3) / 1e6, 2),
        "codewords_per_s": round(ws * args.count / (ms / 1e3), 1),
        "ldpc": {"decoded": int((its > 0).sum()), "crc_ok": int(ok[its > 0].sum()), "stalled": int((its == -3).sum()),
                 "capped": int((its == -1).sum()), "mean_iterations": round(float(lz.iterations_run(its, batch["rates"], MAX_ITER, STALL_IT).mean()), 3),
                 "edge_updates_per_step": edges, "edge_updates_per_s": round(edges / (launch_ms / 1e3), 1),
                 "autotune": tune},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 5),
                     "traffic": None if traffic is None else int(traffic), "peak_source": peak_src,
                     "kernel": "ldpc_decode_kernel<7/8,3/4,2/3,1/2> (the 4 launches of a step)",
                     "note": "not HBM bound: the min-sum minima issue on the ALU pipe (every min/max form does on sm_103a); "
                             "int_op is its roofline",
                     "int_op": int_op_roofline(edges, launch_ms, sm_mhz, sms),
                     "alu_pipe": {"active_frac": 0.856, "measured": False,
                                  "kernel": "ldpc_decode_kernel 7/8 code (41% of a step), 2 warps a codeword, pair form with the loop",
                                  "source": "imported from one ncu capture (sm__pipe_alu_cycles_active, profiles/ldpc_decode_65536cw.md, "
                                            "python bench.py --ldpc-variants --count 16384), not measured in this run"}},
        "gpu_launches": launches,
        "clocks": clocks,
    }
    if e2e:
        out["e2e"] = e2e
    if noalloc:
        out["ldpc"]["noalloc"] = noalloc
    if not args.no_receiver:
        out["receiver"] = bench_receiver(args, stream)
        out["registration"] = {"anchor_search": bench_anchor(args, stream), "refinement": bench_refinement(args, stream),
                               "format_word": bench_fmt_word(args, stream), "border_nodes": bench_border_nodes(args, stream)}
        out["sender"] = bench_encoder(args, stream)
        out["ingest"] = bench_ingest(args, stream)
        out["receiver"]["multistream"] = bench_multistream(args, stream)
    if ws == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        v, dt, kind, (cb, ci, co) = cpu_decode(batch, threads, args.count, outputs=True)
        out["cpu_baseline"] = {"value": round(v, 4), "unit": UNIT, "cores": threads, "kind": kind,
                               "sample": "the whole %d-codeword batch once (%.1f s wall on %d threads)" % (args.count, dt, threads)}
        est = reference_estimate(v, kind)
        if est:
            out["cpu_baseline"]["reference_estimate"] = est
        # the CPU decoder's outputs for every codeword of the batch against the GPU's: bits, iterations, CRC verdicts
        out["ldpc"]["bit_exact_full_batch"] = bool(np.array_equal(ci, its) and np.array_equal(co, ok) and np.array_equal(cb, bits_dev))
        out["ldpc"]["full_batch_checked_against"] = "the CPU decoder of cpu_baseline (%s), all %d codewords" % (kind, args.count)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
