"""Integer float/double conversions of the slicing and tridiagonalisation kernels
(csrc/dfbits.cuh), checked bit for bit against IEEE round-to-nearest-even on the
CPU: the header is compiled with g++ into a small driver."""
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("dfbits") / "dfbits_driver")
    subprocess.run([gxx, "-O2", "-std=c++17", "-o", exe, os.path.join(HERE, "native", "dfbits_driver.cpp")],
                   check=True)
    return exe


def _run(exe, mode, payload):
    out = subprocess.run([exe, mode], input=payload.tobytes(), capture_output=True, check=True).stdout
    return out


def _split_cases(rng):
    xs = [rng.standard_normal(20000) * np.exp2(rng.integers(-80, 128, 20000)).astype(np.float64)]
    # values that are exactly halfway between two floats (ties to even) and just beside them
    q = rng.integers(1 << 23, 1 << 24, 4000).astype(np.float64)
    e = rng.integers(-70, 100, 4000)
    for off in (0.5, 0.5 - 2.0 ** -29, 0.5 + 2.0 ** -29):
        xs.append(np.ldexp(q + off, e - 23) * rng.choice([-1.0, 1.0], 4000))
    # just below powers of two (the head rounds up to the next exponent)
    e2 = rng.integers(-70, 126, 2000)
    xs.append(np.ldexp(1.0 - 2.0 ** -53 * rng.integers(1, 1 << 20, 2000), e2))
    # values exactly representable as floats (zero tail), tails with ties at the tail's precision
    xs.append(rng.standard_normal(2000).astype(np.float32).astype(np.float64))
    t = (rng.integers(1 << 23, 1 << 24, 2000).astype(np.float64) * 2.0 ** -24
         + (rng.integers(1 << 23, 1 << 24, 2000) * 2 + 1).astype(np.float64) * 2.0 ** -54)
    xs.append(t * rng.choice([-1.0, 1.0], 2000))
    # range edges: inside and outside [2^-74, 2^127), zeros, denormals, inf, nan
    edge = [0.0, -0.0, 2.0 ** -74, -(2.0 ** -74), 2.0 ** -74 * (1 - 2.0 ** -53), np.nextafter(2.0 ** 127, 0),
            2.0 ** 127, 2.0 ** -1074, 1e-320, np.inf, -np.inf, np.nan, 1.0, -1.0, 3.0, 2.0 ** 126 * 1.999999]
    xs.append(np.array(edge))
    return np.concatenate(xs).astype(np.float64)


def test_split_matches_ieee_rounding(driver):
    rng = np.random.default_rng(7)
    x = _split_cases(rng)
    out = np.frombuffer(_run(driver, "split", x), dtype=np.uint32).reshape(-1, 3)
    ok = out[:, 0].astype(bool)
    ax = np.abs(x)
    covered = (ax == 0) | ((ax >= 2.0 ** -74) & (ax < 2.0 ** 127))
    covered &= np.isfinite(x)
    assert np.array_equal(ok, covered)
    with np.errstate(over="ignore", invalid="ignore"):
        hi = x.astype(np.float32)
        lo = (x - hi.astype(np.float64)).astype(np.float32)
    assert np.array_equal(out[ok, 1], hi[ok].view(np.uint32))
    assert np.array_equal(out[ok, 2], lo[ok].view(np.uint32))


def test_scaled_rint_matches_rounding(driver):
    rng = np.random.default_rng(9)
    n = 20000
    x = rng.standard_normal(n) * np.exp2(rng.integers(-60, 60, n).astype(np.float64))
    sh = rng.integers(-20, 100, n)
    # ties: odd multiples of 1/2 after scaling, and values just beside them
    k = rng.integers(-(1 << 40), 1 << 40, 3000).astype(np.float64)
    e = rng.integers(-30, 30, 3000)
    xt = np.concatenate([np.ldexp(k + 0.5, e), np.ldexp(k + 0.5, e) * (1 + 2.0 ** -52)])
    st = np.concatenate([-e, -e])
    edge = np.array([0.0, -0.0, 0.5, -0.5, 1.5, 2.5, 2.0 ** -1074, 1e-310, np.inf, -np.inf, np.nan,
                     2.0 ** 61, 2.0 ** 62, np.nextafter(2.0 ** 62, 0), 0.49999999999999994])
    x = np.concatenate([x, xt, edge])
    sh = np.concatenate([sh, st, np.zeros(len(edge), dtype=np.int64)])
    payload = np.zeros(len(x), dtype=[("x", "<f8"), ("sh", "<i8")])
    payload["x"], payload["sh"] = x, sh
    out = np.frombuffer(_run(driver, "rint", payload), dtype=np.int64).reshape(-1, 2)
    ok = out[:, 0].astype(bool)
    with np.errstate(over="ignore", invalid="ignore"):
        y = np.ldexp(x, sh)
        covered = np.isfinite(x) & ((x == 0) | (np.abs(x) >= 2.0 ** -1022)) & (np.abs(y) < 2.0 ** 62)
    assert np.array_equal(ok, covered)
    want = np.rint(y[ok]).astype(np.int64)
    assert np.array_equal(out[ok, 1], want)


def test_absmax_bits(driver):
    rng = np.random.default_rng(10)
    x = rng.standard_normal(5000) * np.exp2(rng.integers(-300, 300, 5000).astype(np.float64))
    x[17] = np.nan
    m = np.frombuffer(_run(driver, "absmax", x), dtype=np.uint64)[0]
    assert m.view(np.float64) == np.nanmax(np.abs(x))
    x[23] = -np.inf
    m = np.frombuffer(_run(driver, "absmax", x), dtype=np.uint64)[0]
    assert m.view(np.float64) == np.inf
