"""shapes_sincos: correctly rounded sine and cosine (CPU checks through the oracle library).

The reference builds rotations from libm's cos and sin (shapes/src/Physics/Linear.hs:353-357);
the CUDA step and the oracle share shapes_sincos, whose results are the correctly rounded
values.  These tests check it against exact arithmetic (mpmath), check that its fast phase
never decides a different double than its accurate phase, and record how often the host libm
differs from it.
"""
from __future__ import annotations

import importlib.util
import math
import struct
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
CSRC = ROOT / "shapes_gb300" / "csrc"


@pytest.fixture(scope="module")
def O(oracle_lib):
    return oracle_lib


def _gen_module():
    spec = importlib.util.spec_from_file_location("gen_sincos_tables", CSRC / "gen_sincos_tables.py")
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def test_tables_header_is_generated():
    """The committed constants are exactly what the generator writes."""
    assert _gen_module().generate() == (CSRC / "shapes_sincos_tables.h").read_text()


def _cr(fn, x: float) -> float:
    """fn(x) correctly rounded to a double (300-bit evaluation, then round to nearest)."""
    mpmath = pytest.importorskip("mpmath")
    with mpmath.workprec(320):
        v = fn(mpmath.mpf(x))
    with mpmath.workprec(53):
        r = +v
    return float(r)


def _args():
    rng = np.random.default_rng(42)
    parts = [
        rng.uniform(-np.pi / 4, np.pi / 4, 400),
        rng.uniform(-10, 10, 800),
        rng.uniform(-1000, 1000, 300),
        rng.uniform(-65536, 65536, 200),
        np.exp(rng.uniform(np.log(1e-9), np.log(1e-6), 100)),
        np.exp(rng.uniform(np.log(6.6e4), np.log(1e300), 200)) * rng.choice([-1, 1], 200),
        # doubles nearest to multiples of pi/2 and of pi/512 (deep cancellation in the reduction)
        np.array([k * math.pi / 2 for k in range(1, 60)]),
        np.array([k * math.pi / 512 for k in range(1, 200, 7)]),
        np.array([6381956970095103.0 * 2.0 ** 797, 5706131972219997.0 * 2.0 ** -30, 22.0, 355.0, 103993.0,
                  1.7976931348623157e308]),
        np.array([float.fromhex(h) for h in ("0x1.921fb54442d18p+0", "0x1.921fb54442d18p+1", "0x1.921fb54442d18p+2",
                                             "0x1.921fb54442d18p-1", "0x1p-27", "0x1.0000000000001p-27",
                                             "0x1.fffffffffffffp-28", "0x1p16", "0x1.fffffffffffffp15")]),
    ]
    return np.concatenate(parts)


def test_correctly_rounded_against_exact(O):
    mpmath = pytest.importorskip("mpmath")
    x = _args()
    s, c = O.sincos(x)
    bad = []
    for k, xv in enumerate(x):
        es, ec = _cr(mpmath.sin, float(xv)), _cr(mpmath.cos, float(xv))
        if s[k] != es or c[k] != ec:
            bad.append((float(xv).hex(), s[k], es, c[k], ec))
    assert not bad, bad[:5]


def test_fast_phase_error_bound(O):
    """The fast phase's double-double is within 2^-67 relative of the exact value
    (the rounding test assumes 2^-65), wherever it does not decline."""
    mpmath = pytest.importorskip("mpmath")
    rng = np.random.default_rng(7)
    x = np.concatenate([rng.uniform(-10, 10, 1500), rng.uniform(-65536, 65536, 500),
                        np.array([k * math.pi / 512 for k in range(1, 1024, 3)])])
    out, ok = O.sincos_phase(x, 1)
    worst = 0.0
    with mpmath.workprec(320):
        for k in np.nonzero(ok)[0]:
            xv = mpmath.mpf(float(x[k]))
            for (hi, lo), ex in (((out[k, 0], out[k, 1]), mpmath.sin(xv)), ((out[k, 2], out[k, 3]), mpmath.cos(xv))):
                err = abs((mpmath.mpf(hi) + mpmath.mpf(lo)) - ex) / abs(ex)
                worst = max(worst, float(err))
    assert worst < 2.0 ** -67, math.log2(worst)


def test_fast_phase_never_disagrees_with_accurate_phase(O):
    """Over 2 x 10^6 arguments: the full function (fast phase + rounding test,
    accurate phase where the test fails) equals the accurate phase alone."""
    rng = np.random.default_rng(3)
    x = np.concatenate([rng.uniform(-10, 10, 10 ** 6), rng.uniform(-np.pi / 4, np.pi / 4, 5 * 10 ** 5),
                        rng.uniform(-65536, 65536, 5 * 10 ** 5)])
    s, c = O.sincos(x)
    acc, _ = O.sincos_phase(x, 0)
    assert np.array_equal(s.view(np.int64), acc[:, 0].view(np.int64))
    assert np.array_equal(c.view(np.int64), acc[:, 2].view(np.int64))


def test_special_values(O):
    x = np.array([0.0, -0.0, 5e-324, -5e-324, 1e-310, 1e-20, -1e-20, np.inf, -np.inf, np.nan])
    s, c = O.sincos(x)
    assert struct.pack("<d", s[0]) == struct.pack("<d", 0.0) and struct.pack("<d", s[1]) == struct.pack("<d", -0.0)
    assert np.array_equal(s[2:7], x[2:7]) and np.all(c[:7] == 1.0)
    assert np.all(np.isnan(s[7:])) and np.all(np.isnan(c[7:]))


def test_host_libm_agreement_is_recorded(O):
    """The host libm (what the reference calls) agrees with the correctly rounded
    values on all but a small fraction of arguments; every disagreement checked
    here is the libm's rounding error, not ours."""
    mpmath = pytest.importorskip("mpmath")
    x = np.random.default_rng(5).uniform(-10, 10, 10 ** 6)
    ns, nc, na, bad = O.sincos_vs_libm(x, cap=50)
    assert ns + nc < 0.01 * len(x)
    assert na < 0.002 * len(x)  # accurate-phase calls
    s, c = O.sincos(bad)
    for k, xv in enumerate(bad):
        assert s[k] == _cr(mpmath.sin, float(xv)) and c[k] == _cr(mpmath.cos, float(xv))
    print(f"host libm vs shapes_sincos over {len(x)} arguments in [-10, 10]: {ns} sin and {nc} cos differ; "
          f"accurate phase used {na} times")
