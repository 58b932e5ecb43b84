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


def test_device_acos_bound_matches_host_build(tmp_path):
    """The float pass's acos bound: the device build gives the host build's bits (same operations, directed
    rounding by intrinsics instead of the FPU mode)."""
    dev = test_acos.build_bound_harness(tmp_path, device=True)
    host = test_acos.build_bound_harness(tmp_path, device=False)
    bits = test_acos.bound_inputs()
    assert (test_acos.bound_rows(dev, bits) == test_acos.bound_rows(host, bits)).all()


def test_device_acos_bound_sound_on_every_float(tmp_path):
    """Every float of [-1, 1] (2,130,706,434 arguments, about a second on the device): lower <= acos rounded
    down and upper >= acos rounded up, at most 8 units apart."""
    dev = test_acos.build_bound_harness(tmp_path, device=True)
    checked, violations, max_w, mean_w = test_acos.bound_sweep(dev, 1)
    assert checked == 2_130_706_434 and violations == 0
    assert max_w <= 8 and mean_w < 3.0
