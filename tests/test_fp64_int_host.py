"""The integer-pipe binary64 addition (add_rn_int, shapes_gb300/csrc/fp64_ops.cuh)
run on the host against the host's own IEEE addition: the same integer steps
the kernels run, checked without a GPU (the probe library loads on CPU)."""
import ctypes

import pytest


@pytest.fixture(scope="module")
def probe(built):
    from shapes_gb300 import build as B

    lib = ctypes.CDLL(str(B.PROBE_LIB))
    lib.shapes_probe_add_check_host.argtypes = [ctypes.c_ulonglong, ctypes.c_ulonglong,
                                                ctypes.POINTER(ctypes.c_ulonglong), ctypes.POINTER(ctypes.c_double)]
    return lib


@pytest.mark.parametrize("seed", [1, 2])
def test_add_rn_int_on_host(probe, seed):
    bad = ctypes.c_ulonglong()
    first = (ctypes.c_double * 2)()
    assert probe.shapes_probe_add_check_host(20_000_000, seed, ctypes.byref(bad), first) == 0
    assert bad.value == 0, f"{bad.value} mismatches, first a={first[0]!r} b={first[1]!r}"
