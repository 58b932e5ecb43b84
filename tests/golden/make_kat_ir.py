#!/usr/bin/env python3
"""Write the known-answer test systems of kat_systems.cpp as lemma IR files into tests/golden/kat/.

The systems are compiled with this repository's front end (include/ivarp) and run with SID_EXPORT_DIR
set, so run_prover writes each compiled IR instead of proving. The file names below follow the call
order in kat_systems.cpp. The GPU build compiles kernels for every IR in tests/golden/kat/.
"""
import os
import re
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.abspath(os.path.join(HERE, "..", ".."))
NAMES = ["expected_critical_f64", "expected_critical_f32", "expected_critical2_f64", "expected_critical2_f32",
         "pos_neg1_sat", "pos_neg1_unsat", "pos_neg2_sat", "pos_neg2_unsat",
         "run_prover_sat_f64", "run_prover_unsat_f64", "run_prover_sat_f32", "run_prover_unsat_f32"]


def main():
    out = os.path.join(HERE, "kat")
    os.makedirs(out, exist_ok=True)
    tmp = tempfile.mkdtemp(prefix="sid_kat_")
    try:
        exe = os.path.join(tmp, "kat_systems")
        subprocess.run(["g++", "-std=c++17", "-O1", "-I" + os.path.join(REPO, "include"),
                        os.path.join(HERE, "kat_systems.cpp"),
                        os.path.join(REPO, "squares-in-disk_gb300", "lemmas", "export_stub.cpp"),
                        "-o", exe, "-lpthread"], check=True)
        ir = os.path.join(tmp, "ir")
        os.makedirs(ir)
        subprocess.run([exe], env=dict(os.environ, SID_EXPORT_DIR=ir), check=True)
        files = sorted(os.listdir(ir))
        assert len(files) == len(NAMES), files
        for name, fn in zip(NAMES, files):
            text = open(os.path.join(ir, fn)).read()
            text = re.sub(r"^name .*$", "name " + name, text, count=1, flags=re.M)
            with open(os.path.join(out, name + ".sidir"), "w") as f:
                f.write(text)
            print(os.path.join(out, name + ".sidir"))
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
