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
    # bundles (several lemmas proved by one persistent kernel): bundles.txt beside the IR files
    bundle_files = sorted({os.path.join(os.path.dirname(p), "bundles.txt") for p in usable} |
                          {os.path.join(d, "bundles.txt") for d in extra_ir_dirs})
    bundle_files = [b for b in bundle_files if os.path.exists(b)]
    bundle_args = [x for b in bundle_files for x in ("--bundles", b)]
    subprocess.run([sys.executable, os.path.join(CSRC, "codegen.py"), "--out", GEN, *bundle_args, *usable], check=True,
                   stdout=subprocess.DEVNULL if not verbose else None)
    gen_units = sorted(glob.glob(os.path.join(GEN, "lemma_*.cu")))
    wanted = {os.path.join(GEN, "lemma_" + _ns(p) + ".cu") for p in usable}
    for stale in set(gen_units) - wanted:
        os.remove(stale)
    gen_units = sorted(wanted)
    wanted_bundles = {os.path.join(GEN, "bundle_%s.cu" % name) for b in bundle_files for name, _ in codegen.read_bundles(b)}
    for stale in set(glob.glob(os.path.join(GEN, "bundle_*.cu"))) - wanted_bundles:
        os.remove(stale)
    # separate compilation (-rdc) for the bundle units and the lemma units they call into, which export their
    # proof-loop parts; a device-link step resolves those calls. Their registers are capped like the one-proof
    # loop kernel's, so the bundle kernel keeps its residency.
    parts = {os.path.join(GEN, "bpart_lemma_" + _ns(x) + ".cu") for b in bundle_files for _, slugs in codegen.read_bundles(b)
             for x in slugs}
    for stale in set(glob.glob(os.path.join(GEN, "bpart_*.cu"))) - parts:
        os.remove(stale)
    part_deps = {p: [os.path.join(GEN, os.path.basename(p)[len("bpart_"):])] for p in parts}
    unit_flags = {u: ["-rdc=true"] for u in wanted_bundles}
    unit_flags.update({u: ["-rdc=true", "-maxrregcount=%d" % _loop_register_cap()] for u in parts})
    units = sorted(parts) + gen_units + sorted(wanted_bundles) + [os.path.join(GEN, "registry.cu"),
                                                                  os.path.join(CSRC, "engine.cu"),
                                                                  os.path.join(CSRC, "noalloc.cu")]
    headers = sorted(glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.hpp")) +
                     [os.path.join(REPO, "include", "sid.h")])

    def compile_unit(src):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        stamp_file = obj + ".stamp"
        flags = NVCC_FLAGS + unit_flags.get(src, [])
        stamp = _stamp([src] + part_deps.get(src, []) + headers, flags)
        if os.path.exists(obj) and os.path.exists(stamp_file) and open(stamp_file).read() == stamp:
            return obj
        cmd = [nvcc(), *flags, "-c", src, "-o", obj]
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
    rdc_objs = [o for u, o in zip(units, objs) if u in unit_flags]
    if rdc_objs:
        dlink = os.path.join(BUILD, "device_link.o")
        dlink_stamp = _stamp(rdc_objs, ["dlink"])
        if not (os.path.exists(dlink) and os.path.exists(dlink + ".stamp") and open(dlink + ".stamp").read() == dlink_stamp):
            cmd = [nvcc(), "-dlink", "-gencode", "arch=compute_103a,code=sm_103a", "-Xcompiler", "-fPIC", *rdc_objs,
                   "-o", dlink]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError("device link failed:\n%s\n%s" % (r.stdout, r.stderr))
            with open(dlink + ".stamp", "w") as f:
                f.write(dlink_stamp)
        objs = objs + [dlink]
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


def _loop_register_cap():
    """Registers per thread of the proof-loop kernels: the bundle kernel is compiled for SID_LOOP_MIN_BLOCKS resident
    128-thread blocks per SM (4 unless a tuning build defines it), and the separately compiled parts it calls must
    not use more (65,536 registers per SM, allocated in groups of 8)."""
    blocks = 4
    for d in NVCC_FLAGS:
        if d.startswith("-DSID_LOOP_MIN_BLOCKS="):
            blocks = int(d.split("=", 1)[1])
    return min(255, 65536 // (128 * max(blocks, 1))) // 8 * 8


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
