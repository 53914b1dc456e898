"""The exact binary64 helpers used by the kernels against the hardware IEEE
operations they replace (integer-pipe comparisons, x + 0.0, and division by a
precomputed reciprocal with Markstein's correction)."""
import ctypes
import math
import struct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def probe(built):
    import torch

    torch.cuda.set_device(0)
    from shapes_gb300 import build as B

    lib = ctypes.CDLL(str(B.PROBE_LIB))
    lib.shapes_probe_div_check.argtypes = [ctypes.c_ulonglong, ctypes.c_ulonglong,
                                           ctypes.POINTER(ctypes.c_ulonglong), ctypes.POINTER(ctypes.c_double)]
    lib.shapes_probe_cmp_check.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.c_int,
                                           ctypes.POINTER(ctypes.c_ulonglong)]
    lib.shapes_probe_mul_check.argtypes = lib.shapes_probe_div_check.argtypes
    lib.shapes_probe_mul_rate.argtypes = [ctypes.POINTER(ctypes.c_double)]
    lib.shapes_probe_add_check.argtypes = lib.shapes_probe_div_check.argtypes
    lib.shapes_probe_split_rates.argtypes = [ctypes.POINTER(ctypes.c_double)]
    return lib


@pytest.mark.parametrize("seed", [11, 12, 13, 14])
def test_div_rn_matches_hardware_division(probe, seed):
    bad = ctypes.c_ulonglong()
    first = (ctypes.c_double * 2)()
    assert probe.shapes_probe_div_check(1 << 28, seed, ctypes.byref(bad), first) == 0
    assert bad.value == 0, f"{bad.value} mismatches, first a={first[0]!r} b={first[1]!r}"


def test_integer_comparisons_match_ieee(probe):
    specials = [0.0, -0.0, 1.0, -1.0, math.inf, -math.inf, math.nan, -math.nan, 5e-324, -5e-324,
                2.2250738585072014e-308, 1.7976931348623157e308, -1.7976931348623157e308, 0.5, 2.0, 3.0,
                -3.0, 1e-300, -1e300, 1.0000000000000002, 0.9999999999999999]
    rng = np.random.default_rng(0)
    rnd = rng.standard_normal(200) * 10.0 ** rng.integers(-300, 300, 200)
    vals = np.array(specials + list(rnd) + [struct.unpack("<d", struct.pack("<Q", 0x7ff8000000000001))[0]])
    bad = ctypes.c_ulonglong()
    assert probe.shapes_probe_cmp_check(vals.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), len(vals),
                                        ctypes.byref(bad)) == 0
    assert bad.value == 0


@pytest.mark.parametrize("seed", [21, 22, 23, 24])
def test_integer_pipe_multiply_matches_hardware(probe, seed):
    bad = ctypes.c_ulonglong()
    first = (ctypes.c_double * 2)()
    assert probe.shapes_probe_mul_check(1 << 28, seed, ctypes.byref(bad), first) == 0
    assert bad.value == 0, f"{bad.value} mismatches, first a={first[0]!r} b={first[1]!r}"


def test_integer_pipe_multiply_rate(probe):
    rates = (ctypes.c_double * 2)()
    assert probe.shapes_probe_mul_rate(rates) == 0
    assert rates[0] > 0 and rates[1] > 0
    print(f"multiplies/s: hardware {rates[0]:.3e}, integer pipe {rates[1]:.3e}")


@pytest.mark.parametrize("seed", [31, 32, 33, 34])
def test_integer_pipe_add_matches_hardware(probe, seed):
    bad = ctypes.c_ulonglong()
    first = (ctypes.c_double * 2)()
    assert probe.shapes_probe_add_check(1 << 28, seed, ctypes.byref(bad), first) == 0
    assert bad.value == 0, f"{bad.value} mismatches, first a={first[0]!r} b={first[1]!r}"


def test_split_rates(probe):
    """Sums and products per second with chains on the FP64 pipe, on the
    integer pipe (add_rn_int / mul_rn_int) and split 4 + 4 in the same warps."""
    r = (ctypes.c_double * 6)()
    assert probe.shapes_probe_split_rates(r) == 0
    assert all(x > 0 for x in r)
    print(f"adds/s: FP64 {r[0]:.3e}, integer {r[1]:.3e}, split {r[2]:.3e}; "
          f"products/s: FP64 {r[3]:.3e}, integer {r[4]:.3e}, split {r[5]:.3e}")
