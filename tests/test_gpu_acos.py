"""GPU test of the directed arc cosine: the device build of squares-in-disk_gb300/csrc/acos.cuh (one argument
per thread, tests/acos_check.cpp compiled with nvcc for sm_103a and the engine's floating-point flags) must
give the exact downward and upward roundings recorded in tests/golden/acos_cases.txt (from 300-bit mpmath;
the reference rounds acos with MPFR, ivarp/src/interval_acos.cpp:29-34), including the structured arguments
that need the four-limb evaluation.
"""
import pytest

import test_acos

pytestmark = pytest.mark.gpu


def test_device_acos_matches_golden_cases(tmp_path):
    exe = test_acos.build_harness(tmp_path, device=True)
    assert test_acos.check_golden(exe) > 1500
