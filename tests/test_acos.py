"""Correctly rounded directed arc cosine: the device algorithm (csrc/acos.cuh, built for the host by
tests/acos_check.cpp) and the oracle's independent version (oracle/acos_cr.hpp) against mpmath at
300 bits.

The reference rounds acos with MPFR at the number type's precision (ivarp/src/interval_acos.cpp:29-34):
downward and upward results must be the neighbours around the exact value, bit for bit. Inputs cover
the three branches of the device method (|x| <= 1/2, x > 1/2, x < -1/2), their boundaries, arguments
next to +-1 (results down to 2^-26), tiny and subnormal arguments, float inputs, and the domain edges.
"""
import math
import os
import struct
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(REPO, "squares-in-disk_gb300", "csrc")
GOLDEN = os.path.join(HERE, "golden", "acos_cases.txt")


def build_harness(out_dir, device=False):
    """Compile tests/acos_check.cpp for the host (g++) or for the GPU (nvcc, sm_103a, the engine's FP flags)."""
    exe = os.path.join(str(out_dir), "acos_check_dev" if device else "acos_check")
    src = os.path.join(HERE, "acos_check.cpp")
    if device:
        cmd = ["nvcc", "-std=c++17", "-O3", "-x", "cu", "-gencode", "arch=compute_103a,code=sm_103a", "--fmad=false",
               "--ftz=false", "--prec-div=true", "--prec-sqrt=true", "-I", CSRC, src, "-o", exe]
    else:
        cmd = ["g++", "-std=c++17", "-O2", "-I", CSRC, src, "-o", exe]
    subprocess.run(cmd, check=True)
    return exe


def run_lines(exe, kinds, xs):
    lines = "".join("%s %s\n" % (k, struct.pack(">d", float(x)).hex()) for k, x in zip(kinds, xs))
    out = subprocess.run([exe], input=lines, capture_output=True, text=True, check=True).stdout.split("\n")
    rows = [l.split() for l in out if l.strip()]
    assert len(rows) == len(xs)
    return rows


def check_golden(exe):
    """Run the harness over tests/golden/acos_cases.txt; returns the number of cases checked."""
    cases = [l.split() for l in open(GOLDEN) if l.strip()]
    kinds = [c[0] for c in cases]
    xs = [struct.unpack(">d", bytes.fromhex(c[1]))[0] for c in cases]
    rows = run_lines(exe, kinds, xs)
    width = {"d": 16, "f": 8}
    for c, r in zip(cases, rows):
        w = width[c[0]]
        assert (r[0].zfill(w), r[1].zfill(w)) == (c[2], c[3]), c
        if c[1] != "3ff0000000000000":
            assert r[3] == "1", c   # four limbs always decide
    return len(cases)


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    return build_harness(tmp_path_factory.mktemp("acos"))


def _run(exe, kind, xs):
    return run_lines(exe, [kind] * len(xs), xs)


def test_device_acos_host_build_matches_golden_cases(harness):
    assert check_golden(harness) > 1500


def _expected(x, digits):
    """(downward, upward) rounding of acos(x) to a binary format with `digits` bits, via 300-bit mpmath."""
    mpmath = _mp()
    with mpmath.workprec(300):
        v = mpmath.acos(mpmath.mpf(x))
        if v == 0:
            return 0.0, 0.0
        if digits == 53:
            d = float(v)
            if mpmath.mpf(d) > v:
                d = math.nextafter(d, -math.inf)
            assert mpmath.mpf(d) < v
            return d, math.nextafter(d, math.inf)
        f = np.float32(float(v))
        if mpmath.mpf(float(f)) > v:
            f = np.nextafter(f, np.float32(-np.inf))
        assert mpmath.mpf(float(f)) < v
        return float(f), float(np.nextafter(f, np.float32(np.inf)))


def _mp():
    return pytest.importorskip("mpmath")


def _inputs_double():
    rng = np.random.default_rng(20201123)
    xs = [0.0, -0.0, 0.5, -0.5, 1.0, -1.0, 5e-324, -5e-324, 2.0 ** -1022, 1e-300, 2.0 ** -74, 2.0 ** -75,
          0.25, -0.25, 0.75, -0.75, 1.0 - 2.0 ** -53, -1.0 + 2.0 ** -53, 0.5 + 2.0 ** -53, 0.5 - 2.0 ** -54,
          -0.5 - 2.0 ** -53, math.cos(1.0), math.cos(2.0), 1.0 / 3.0]
    xs += list(rng.uniform(-1.0, 1.0, 4000))
    for sign in (1.0, -1.0):
        xs += [sign * (1.0 - k * 2.0 ** -53) for k in range(1, 40)]
        xs += [sign * (1.0 - 2.0 ** -e) for e in range(1, 54)]
        xs += list(sign * (1.0 - np.exp2(-rng.uniform(1.0, 53.0, 600))))
        xs += list(sign * np.exp2(-rng.uniform(1.0, 1074.0, 300)))
        xs += list(sign * (0.5 + rng.integers(-2000, 2000, 200) * 2.0 ** -53))
    return [float(x) for x in xs]


def _inputs_structured():
    """x = 1 - c^2 2^-(2d+1): then sqrt(2(1-x)) = c 2^-d is dyadic and acos(x) = c 2^-d (1 + (1-x)/12 + ...)
    lies unusually close to a double, so the two-limb evaluation cannot always decide the rounding."""
    xs = []
    for c in range(1, 200):
        for k in range(1, 54):
            eps = c * c * 2.0 ** -k
            if eps < 0.5 and (eps / 2.0 ** -53).is_integer():
                xs.append(1.0 - eps)
    return sorted(set(xs))


def _inputs_float():
    rng = np.random.default_rng(7)
    xs = list(rng.uniform(-1.0, 1.0, 1500).astype(np.float32))
    xs += [np.float32(1.0) - np.float32(k) * np.float32(2.0 ** -24) for k in range(1, 30)]
    xs += [-(np.float32(1.0) - np.float32(k) * np.float32(2.0 ** -24)) for k in range(1, 30)]
    xs += [np.float32(0.5), np.float32(-0.5), np.float32(0.0), np.float32(2.0 ** -149)]
    return [float(x) for x in xs]


def _check_double(harness, xs):
    undecided2 = []
    for x, (rd, ru, dec2, dec4, rd4) in zip(xs, _run(harness, "d", xs)):
        want_rd, want_ru = _expected(x, 53)
        got_rd = struct.unpack(">d", bytes.fromhex(rd.zfill(16)))[0]
        got_ru = struct.unpack(">d", bytes.fromhex(ru.zfill(16)))[0]
        assert (got_rd, got_ru) == (want_rd, want_ru), x
        if x != 1.0:
            assert dec4 == "1", x   # four limbs always decide
            assert struct.unpack(">d", bytes.fromhex(rd4.zfill(16)))[0] == want_rd, x
            if dec2 != "1":
                undecided2.append(x)
    return undecided2


def test_device_acos_double_correctly_rounded(harness):
    assert _check_double(harness, _inputs_double()) == []   # two limbs decide every generic argument


def test_device_acos_structured_hard_cases_use_four_limbs(harness):
    xs = _inputs_structured()
    undecided2 = _check_double(harness, xs)
    assert 1.0 - 9 * 2.0 ** -49 in undecided2   # the fallback path is exercised and correct
    assert len(undecided2) < len(xs) // 10


def test_device_acos_float_correctly_rounded(harness):
    xs = _inputs_float()
    rows = _run(harness, "f", xs)
    for x, (rd, ru, dec2, dec4, rd4) in zip(xs, rows):
        want_rd, want_ru = _expected(x, 24)
        got_rd = struct.unpack(">f", bytes.fromhex(rd.zfill(8)))[0]
        got_ru = struct.unpack(">f", bytes.fromhex(ru.zfill(8)))[0]
        assert (got_rd, got_ru) == (want_rd, want_ru), x
        if x != 1.0:
            assert struct.unpack(">f", bytes.fromhex(rd4.zfill(8)))[0] == want_rd, x


def test_device_acos_domain(harness):
    xs = [1.0 + 2.0 ** -52, -1.0 - 2.0 ** -52, 2.0, float("inf"), float("-inf"), float("nan")]
    for rd, ru, *_ in _run(harness, "d", xs):
        assert math.isnan(struct.unpack(">d", bytes.fromhex(rd.zfill(16)))[0])
        assert math.isnan(struct.unpack(">d", bytes.fromhex(ru.zfill(16)))[0])
    rd, ru, *_ = _run(harness, "d", [1.0])[0]
    assert rd == "0" and ru == "0"   # acos(1) = +0 in both directions


def test_oracle_acos_correctly_rounded(oracle):
    xs = np.array(_inputs_double() + _inputs_structured())
    got_rd = oracle.acos_rounded(xs, False)
    got_ru = oracle.acos_rounded(xs, True)
    for x, a, b in zip(xs, got_rd, got_ru):
        assert (a, b) == _expected(float(x), 53), x
    xf = np.array(_inputs_float(), dtype=np.float32)
    f_rd = oracle.acos_rounded(xf, False, np.float32)
    f_ru = oracle.acos_rounded(xf, True, np.float32)
    for x, a, b in zip(xf, f_rd, f_ru):
        assert (float(a), float(b)) == _expected(float(x), 24), x
    bad = oracle.acos_rounded(np.array([1.5, -1.0000000000000002, np.nan]), True)
    assert np.isnan(bad).all()


# --- the precision form's float-pass bound (acos_bound_f32): sound, a few units wide, same bits in the oracle

def build_bound_harness(out_dir, device=False):
    """Compile tests/acos_bound_check.cpp for the host (g++, directed rounding by the FPU mode) or the GPU."""
    exe = os.path.join(str(out_dir), "acos_bound_check_dev" if device else "acos_bound_check")
    src = os.path.join(HERE, "acos_bound_check.cpp")
    if device:
        cmd = ["nvcc", "-std=c++17", "-O3", "-x", "cu", "-gencode", "arch=compute_103a,code=sm_103a", "--fmad=false",
               "--ftz=false", "--prec-div=true", "--prec-sqrt=true", "-I", CSRC, src, "-o", exe]
    else:
        cmd = ["g++", "-std=c++17", "-O2", "-frounding-math", "-ffp-contract=off", "-I", CSRC, src, "-o", exe]
    subprocess.run(cmd, check=True)
    return exe


def bound_rows(exe, bits):
    out = subprocess.run([exe], input="".join("%08x\n" % int(b) for b in bits), capture_output=True, text=True,
                         check=True).stdout.split()
    return np.array([int(v, 16) for v in out], dtype=np.uint32).reshape(-1, 4)


def bound_sweep(exe, stride):
    out = subprocess.run([exe, "sweep", str(stride)], capture_output=True, text=True, check=True).stdout.split()
    checked, violations, _first, max_w, sum_w = (int(v) for v in out)
    return checked, violations, max_w, sum_w / max(checked, 1)


def bound_inputs():
    """Float bit patterns: the branch boundaries +-1/2, +-1, signed zeros, subnormals, and seeded random floats."""
    rng = np.random.default_rng(11)
    edge = [0x3f000000, 0x3f000001, 0x3effffff, 0xbf000000, 0xbf000001, 0xbeffffff, 0x3f800000, 0xbf800000,
            0x3f7fffff, 0xbf7fffff, 0, 0x80000000, 1, 0x80000001, 0x007fffff, 0x00800000, 0x3e800000]
    rnd = list(rng.integers(0, 0x3f800001, 6000)) + list(0x80000000 | rng.integers(0, 0x3f800001, 6000))
    return np.array(edge + rnd, dtype=np.uint32)


@pytest.fixture(scope="module")
def bound_harness(tmp_path_factory):
    return build_bound_harness(tmp_path_factory.mktemp("acos_bound"))


def test_acos_bound_coefficients_enclose_the_series(bound_harness):
    """The float bounds of c_k = binom(2k, k) / (4^k (2k+1)) used by acos_bound_f32 are the neighbours of c_k,
    and the remainder after 11 terms is below r 2^-28 for r <= 1/2."""
    from fractions import Fraction
    out = subprocess.run([bound_harness, "coef"], capture_output=True, text=True, check=True).stdout.split()
    bounds = np.array([int(v, 16) for v in out], dtype=np.uint32).view(np.float32).reshape(11, 2)
    for k in range(11):
        c = Fraction(math.comb(2 * k, k), 4 ** k * (2 * k + 1))
        f_lo, f_hi = bounds[k]
        assert Fraction(float(f_lo)) <= c <= Fraction(float(f_hi)), k
        assert f_lo == f_hi if Fraction(float(f_lo)) == c else np.nextafter(f_lo, np.float32(2)) == f_hi, k
    c11 = Fraction(math.comb(22, 11), 4 ** 11 * 23)
    assert c11 * Fraction(1, 4 ** 11) / Fraction(3, 4) < Fraction(1, 2 ** 28)


def test_acos_bound_sound_on_a_strided_sweep_of_all_floats(bound_harness):
    checked, violations, max_w, mean_w = bound_sweep(bound_harness, 4099)
    assert checked > 500000 and violations == 0
    assert max_w <= 8 and mean_w < 3.0


def test_acos_bound_edges_and_oracle_restatement(bound_harness, oracle):
    bits = bound_inputs()
    rows = bound_rows(bound_harness, bits)
    lo, hi, rd, ru = (rows[:, i].view(np.float32) for i in range(4))
    assert (lo <= rd).all() and (hi >= ru).all()
    x = bits.view(np.float32)
    assert np.array_equal(oracle.acos_bound_f32(x, False).view(np.uint32), rows[:, 0])
    assert np.array_equal(oracle.acos_bound_f32(x, True).view(np.uint32), rows[:, 1])
    one = int(np.nonzero(bits == 0x3f800000)[0][0])
    assert lo[one] == 0.0 and 0.0 < hi[one] < 1e-40    # acos(1) = 0 is enclosed by a subnormal upper end
