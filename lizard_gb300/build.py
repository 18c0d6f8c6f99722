"""Builds the library in-tree: lizard_gb300/liblizard_gb300.so from csrc/ (CUDA for sm_103a plus host C++).

No cmake: nvcc on each translation unit in parallel, then one link. Objects go to lizard_gb300/_build/.
"""
import concurrent.futures
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "liblizard_gb300.so")
BUILD = os.path.join(HERE, "_build")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code rounds once an operation on every host (gcc contracts a * b + c into one fused operation by default on
# aarch64, not on x86-64), so the library's host-side tables are the same numbers wherever it is built.
COMMON = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-I" + CSRC, "-I" + os.path.join(ROOT, "include")]
# Translation units whose float and double arithmetic must round once an operation, in source order (no fused
# multiply-add): they reproduce the reference's soft values bit for bit.
EXACT = {"demap.cu": ["-fmad=false"], "sample.cu": ["-fmad=false"], "anchor.cu": ["-fmad=false"], "refine.cu": ["-fmad=false"], "ingest.cu": ["-fmad=false"],
         "fmtword.cu": ["-fmad=false"],
         "encode.cu": ["-fmad=false"],
         "mesh.cu": ["-fmad=false"]}


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _newest_input():
    paths = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    return max(os.path.getmtime(p) for p in paths)


def _compile(src, extra):
    obj = os.path.join(BUILD, src + ".o")
    cmd = [NVCC] + COMMON + extra + EXACT.get(src, [])
    if src.endswith(".cu"):
        cmd += ARCH + ["-lineinfo", "-Xptxas", "-v"] if os.environ.get("LIZG_PTXAS_V") else ARCH + ["-lineinfo"]
        cmd += ["-x", "cu"]
    else:
        cmd += ["-x", "c++"]
    cmd += ["-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    return src, obj, r.returncode, r.stdout + r.stderr


def build(force=False, extra=(), verbose=False):
    """Compiles every source and links the shared library. Skips the work when the library is newer than every
    source, unless force. Raises RuntimeError with the compiler's output on failure."""
    if not force and os.path.exists(OUT) and os.path.getmtime(OUT) >= _newest_input():
        return OUT
    os.makedirs(BUILD, exist_ok=True)
    objs = []
    with concurrent.futures.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        for src, obj, rc, log in ex.map(lambda s: _compile(s, list(extra)), sources()):
            if rc != 0:
                raise RuntimeError("compiling %s failed:\n%s" % (src, log))
            if verbose and log.strip():
                print(log)
            objs.append(obj)
    tmp = OUT + ".tmp"
    cmd = [NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart_static", "-lpthread", "-ldl", "-lrt"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("linking failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
