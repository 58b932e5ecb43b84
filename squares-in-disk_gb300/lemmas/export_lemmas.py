#!/usr/bin/env python3
"""Produce the lemma IR files from the reference's unchanged lemma sources.

The reference's src/*.cpp (main.cpp and the nine lemma files) are compiled, unchanged, against this
repository's ivarp front end (include/ivarp) and linked with export_stub.cpp. Run with SID_EXPORT_DIR
set, every run_prover call writes the compiled lemma IR instead of proving. The lemma names printed by
the reference's run_proof ("Starting proof <name>...") are attached to the files in call order.

  python export_lemmas.py [--reference DIR] [--out DIR] [--check]

The reference tree is taken from --reference, else from the environment variable SID_REFERENCE_DIR, else
from the mount point of the machine that holds the reference checkout (reference_dir()).

--check regenerates into a temporary directory and fails if any committed file differs.
This needs the reference sources, so it runs only where they are present.
"""
import argparse
import os
import re
import shutil
import subprocess
import sys
import tempfile
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.abspath(os.path.join(HERE, "..", ".."))
REFERENCE_MOUNT = "/root/reference"   # where the build machine mounts the reference checkout (read-only)


def reference_dir():
    """The reference checkout: SID_REFERENCE_DIR if set, else the build machine's mount point."""
    return os.environ.get("SID_REFERENCE_DIR") or REFERENCE_MOUNT
SOURCES = ["main", "top_packing", "one_subcontainer", "two_subcontainer", "three_subcontainer",
           "four_subcontainer", "five_subcontainer", "six_subcontainer", "seven_subcontainer",
           "more_subcontainers"]

SLUGS = {
    "Top Packing Lemma, statement (1)": "top_packing_1",
    "Top Packing Lemma, statement (2)": "top_packing_2",
    "One Subcontainer Lemma": "one_subcontainer",
    "Two Subcontainer Lemma": "two_subcontainer",
    "Three Subcontainer Lemma": "three_subcontainer",
    "Four Subcontainer Lemma": "four_subcontainer",
    "Five Subcontainers, s_n > sigma": "five_subcontainer",
    "Six Subcontainers, s_n > sigma": "six_subcontainer",
    "Seven Subcontainers, s_n > sigma": "seven_subcontainer",
    ">= 5 Subcontainers, s_n <= sigma, y_3 <= 0": "more_subcontainers_1",
    ">= 5 Subcontainers, s_n <= sigma, y_3 > 0": "more_subcontainers_2",
}


def escape(name):
    out = []
    for ch in name:
        if ch.isalnum() or ch in "_-.,{}><=()":
            out.append(ch)
        else:
            out.append("%%%02X" % ord(ch))
    return "".join(out)


def build_exporter(reference, build_dir):
    os.makedirs(build_dir, exist_ok=True)
    flags = ["-std=c++17", "-O1", "-I" + os.path.join(REPO, "include")]

    def compile_one(src):
        obj = os.path.join(build_dir, os.path.basename(src) + ".o")
        subprocess.run(["g++", *flags, "-c", src, "-o", obj], check=True)
        return obj

    srcs = [os.path.join(reference, "src", s + ".cpp") for s in SOURCES]
    srcs.append(os.path.join(HERE, "export_stub.cpp"))
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        objs = list(ex.map(compile_one, srcs))
    exe = os.path.join(build_dir, "lemma_exporter")
    subprocess.run(["g++", *objs, "-o", exe, "-lpthread"], check=True)
    return exe


def export(reference, out_dir, build_dir):
    exe = build_exporter(reference, build_dir)
    raw = tempfile.mkdtemp(prefix="sid_export_")
    try:
        env = dict(os.environ, SID_EXPORT_DIR=raw)
        proc = subprocess.run([exe], env=env, check=True, capture_output=True, text=True)
        names = re.findall(r"^Starting proof (.*)\.\.\.$", proc.stdout, re.M)
        files = sorted(f for f in os.listdir(raw) if f.endswith(".sidir"))
        if len(names) != len(files):
            raise RuntimeError("expected one IR file per proof: %d names, %d files" % (len(names), len(files)))
        os.makedirs(out_dir, exist_ok=True)
        written = []
        for name, fn in zip(names, files):
            with open(os.path.join(raw, fn)) as f:
                text = f.read()
            text = re.sub(r"^name .*$", "name " + escape(name), text, count=1, flags=re.M)
            dest = os.path.join(out_dir, SLUGS[name] + ".sidir")
            with open(dest, "w") as f:
                f.write(text)
            written.append(dest)
        return written
    finally:
        shutil.rmtree(raw, ignore_errors=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=None)
    ap.add_argument("--out", default=HERE)
    ap.add_argument("--check", action="store_true")
    args = ap.parse_args()
    if args.reference is None:
        args.reference = reference_dir()
    build_dir = os.path.join(HERE, "_build")
    if args.check:
        tmp = tempfile.mkdtemp(prefix="sid_check_")
        try:
            written = export(args.reference, tmp, build_dir)
            bad = []
            for path in written:
                committed = os.path.join(args.out, os.path.basename(path))
                if not os.path.exists(committed) or open(committed).read() != open(path).read():
                    bad.append(os.path.basename(path))
            if bad:
                print("differs:", ", ".join(bad))
                return 1
            print("all %d lemma IR files match" % len(written))
            return 0
        finally:
            shutil.rmtree(tmp, ignore_errors=True)
    for p in export(args.reference, args.out, build_dir):
        print(p)
    return 0


if __name__ == "__main__":
    sys.exit(main())
