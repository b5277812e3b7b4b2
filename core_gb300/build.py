"""Builds the sm_103a estimate-and-mark library in-tree.

``python -m core_gb300.build`` compiles every translation unit under
``core_gb300/csrc`` with nvcc for sm_103a (in parallel) and links
``core_gb300/libsprgb300.so``.  The FP64 parity kernels are compiled with
``-fmad=false`` so their rounding follows the reference's operation order.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libsprgb300.so")
BUILD = os.path.join(HERE, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]

# translation unit -> extra flags
UNITS = {
    "sprg_kernels_f64.cu": ["-fmad=false"],
    "sprg_kernels_f32.cu": [],
    "sprg_capi.cu": [],
    "sprg_noalloc.cu": [],
    "sprg_learned.cu": [],
    "sprg_box.cpp": ["-x", "cu"],
    "sprg_smb.cpp": [],
    "sprg_order.cpp": [],
}


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _compile(unit, extra, verbose):
    src = os.path.join(CSRC, unit)
    obj = os.path.join(BUILD, unit + ".o")
    cmd = [_nvcc()] + ARCH + COMMON + extra + ["-c", src, "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    return unit, obj, r.returncode, r.stdout + r.stderr


def build(verbose=False, force=False):
    """Compile and link; returns the path of the shared library."""
    os.makedirs(BUILD, exist_ok=True)
    units = {u: f for u, f in UNITS.items() if os.path.exists(os.path.join(CSRC, u))}
    srcs = [os.path.join(CSRC, u) for u in units] + [
        os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))
    ] + [os.path.join(ROOT, "include", "spr_gb300.h")]
    if not force and os.path.exists(OUT):
        newest = max(os.path.getmtime(s) for s in srcs)
        if os.path.getmtime(OUT) >= newest:
            return OUT
    with ThreadPoolExecutor(max_workers=len(units)) as ex:
        results = list(ex.map(lambda kv: _compile(kv[0], kv[1], verbose), units.items()))
    failed = [r for r in results if r[2] != 0]
    for unit, _, rc, log in results:
        if log.strip() and (verbose or rc):
            sys.stderr.write(f"--- {unit} ---\n{log}\n")
    if failed:
        raise RuntimeError("nvcc failed for: " + ", ".join(r[0] for r in failed))
    objs = [r[1] for r in results]
    tmp = OUT + ".tmp"
    cmd = [_nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, OUT)
    return OUT


def reference_tree():
    """The SCOREC/core source tree to build the pinning checker from:
    $SPRG_REFERENCE_TREE, else the tree's mount point in the development
    container; None where neither exists (the GPU host)."""
    for cand in (os.environ.get("SPRG_REFERENCE_TREE"), "/root/reference"):
        if cand and os.path.isdir(os.path.join(cand, "mth")):
            return cand
    return None


def build_oracle():
    """Builds the CPU oracle (test infrastructure) and, when the reference
    tree is present on this machine, the checker's copies of the reference:
    its QR alone (oracle/_ref/libmthqr_ref.so) and its whole
    estimate-and-mark path (oracle/_ref/libspr_ref.so), compiled from the
    tree's sources by oracle/Makefile."""
    oracle_dir = os.path.join(ROOT, "oracle")
    subprocess.run(["make", "-s", "-C", oracle_dir], check=True)
    ref = reference_tree()
    if ref:
        jobs = "-j%d" % max(1, os.cpu_count() or 1)
        subprocess.run(["make", "-s", jobs, "-C", oracle_dir, "ref", "refall", "shim", "REF=" + ref], check=True)


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
    build_oracle()
