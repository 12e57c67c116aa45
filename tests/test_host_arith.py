"""The project's own exp (Cody-Waite reduction + Taylor polynomial) and the
float-float ECI dot, built for the host from the same header the kernels use."""

import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def test_expf_error_bound(tmp_path):
    exe = str(tmp_path / "probe")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off",
                    os.path.join(HERE, "host_arith_probe.cc"), "-o", exe], check=True)
    x = np.concatenate([-np.logspace(-8, np.log10(86.9), 4000), [0.0, -1e-30, -87.5, -200.0]])
    out = subprocess.run([exe], input="\n".join(repr(float(np.float32(v))) for v in x),
                         capture_output=True, text=True, check=True).stdout.split()
    got = np.array([float(v) for v in out])
    ref = np.exp(x.astype(np.float32).astype(np.float64))
    ok = x > -87.0
    rel = np.abs(got[ok] - ref[ok]) / ref[ok]
    assert rel.max() < 4e-7, rel.max()
    assert np.all(got[~ok] == 0.0)
    assert got[x == 0.0][0] == 1.0


def _ff_dot(w, dc):
    """Float-float dot in the documented operation order (numpy float32)."""
    f = np.float32
    s, e = f(0), f(0)
    for wf, c in zip(w, dc):
        if c == 0:
            continue
        hi = f(wf)
        lo = f(wf - float(hi))
        c = f(c)
        p = f(hi * c)
        pe = f(float(hi) * float(c) - float(p))  # exact product error
        t = f(s + p)
        z = f(t - s)
        err = f(f(s - f(t - z)) + f(p - z))
        s = t
        e = f(e + f(err + pe))
        e = f(float(lo) * float(c) + float(e))
    return float(s) + float(e)


def test_float_float_dot_within_1e10():
    rng = np.random.default_rng(3)
    for _ in range(2000):
        w = rng.normal(0, 0.02, 27) / rng.integers(1, 25, 27)
        dc = rng.integers(-72, 73, 27) * (rng.random(27) < 0.6)
        exact = float(np.dot(w, dc))
        got = _ff_dot(w, dc)
        assert abs(got - exact) <= 1e-10 * max(abs(exact), 1e-3)
