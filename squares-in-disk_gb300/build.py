#!/usr/bin/env python3
"""Build the GB300 engine library (libsid.so) in-tree.

Steps: generate one CUDA translation unit per lemma IR (csrc/codegen.py), compile every .cu for
sm_103a with nvcc in parallel, link libsid.so into squares-in-disk_gb300/_build/. Rebuilds only what
changed. The floating-point flags keep IEEE semantics (no FMA contraction, no flush-to-zero, IEEE
division and square root); the kernels use directed-rounding intrinsics explicitly.

  python build.py [--ir-dir DIR ...] [--verbose]
"""
import argparse
import glob
import hashlib
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.environ.get("SID_BUILD_DIR") or os.path.join(HERE, "_build")   # another directory for variant builds
GEN = os.path.join(BUILD, "gen")
LIB = os.path.join(BUILD, "libsid.so")

NVCC_FLAGS = [
    "-std=c++17", "-O3", "-lineinfo",
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-Xcompiler", "-fPIC",
    "--fmad=false", "--ftz=false", "--prec-div=true", "--prec-sqrt=true",
    "-I" + CSRC, "-I" + os.path.join(REPO, "include"),
] + os.environ.get("SID_NVCC_DEFINES", "").split()   # e.g. "-DSID_FILTER_MIN_BLOCKS=6" for tuning builds


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def default_ir_files(extra_dirs=()):
    files = sorted(glob.glob(os.path.join(HERE, "lemmas", "*.sidir")))
    for d in extra_dirs:
        files += sorted(glob.glob(os.path.join(d, "*.sidir")))
    return files


def _stamp(paths, flags):
    h = hashlib.sha256()
    for p in paths:
        with open(p, "rb") as f:
            h.update(f.read())
    h.update(" ".join(flags).encode())
    return h.hexdigest()


def build(ir_files=None, extra_ir_dirs=(), verbose=False, jobs=None):
    os.makedirs(GEN, exist_ok=True)
    if ir_files is None:
        ir_files = default_ir_files(extra_ir_dirs)
    sys.path.insert(0, CSRC)
    import codegen  # noqa: E402

    usable = list(ir_files)
    subprocess.run([sys.executable, os.path.join(CSRC, "codegen.py"), "--out", GEN, *usable], check=True,
                   stdout=subprocess.DEVNULL if not verbose else None)
    gen_units = sorted(glob.glob(os.path.join(GEN, "lemma_*.cu")))
    wanted = {os.path.join(GEN, "lemma_" + _ns(p) + ".cu") for p in usable}
    for stale in set(gen_units) - wanted:
        os.remove(stale)
    gen_units = sorted(wanted)
    units = gen_units + [os.path.join(GEN, "registry.cu"), os.path.join(CSRC, "engine.cu"),
                         os.path.join(CSRC, "noalloc.cu")]
    headers = sorted(glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.hpp")) +
                     [os.path.join(REPO, "include", "sid.h")])

    def compile_unit(src):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        stamp_file = obj + ".stamp"
        stamp = _stamp([src] + headers, NVCC_FLAGS)
        if os.path.exists(obj) and os.path.exists(stamp_file) and open(stamp_file).read() == stamp:
            return obj
        cmd = [nvcc(), *NVCC_FLAGS, "-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
        with open(stamp_file, "w") as f:
            f.write(stamp)
        return obj

    with ThreadPoolExecutor(max_workers=jobs or max(2, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_unit, units))
    link_stamp = _stamp(objs, ["link"])
    lib_stamp = LIB + ".stamp"
    if not (os.path.exists(LIB) and os.path.exists(lib_stamp) and open(lib_stamp).read() == link_stamp):
        cmd = [nvcc(), "-shared", "-gencode", "arch=compute_103a,code=sm_103a", "-o", LIB, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
        with open(lib_stamp, "w") as f:
            f.write(link_stamp)
    return LIB


def _ns(path):
    import re
    return re.sub(r"[^A-Za-z0-9_]", "_", os.path.splitext(os.path.basename(path))[0])


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ir-dir", action="append", default=[])
    ap.add_argument("--verbose", action="store_true")
    args = ap.parse_args()
    print(build(extra_ir_dirs=args.ir_dir, verbose=args.verbose))
    return 0


if __name__ == "__main__":
    sys.exit(main())
