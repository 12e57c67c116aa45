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


def test_exp64_restatement_matches_oracle_and_libm(tmp_path, oracle_mod):
    """The FP64 exp of the n-fold rates: the product's host build and the
    oracle's restatement give the same bits, within 1 ulp of libm."""
    exe = str(tmp_path / "probe64")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off",
                    os.path.join(HERE, "host_exp64_probe.cc"), "-o", exe], check=True)
    rng = np.random.default_rng(5)
    x = np.concatenate([-rng.uniform(0, 1, 2000), -rng.uniform(0, 50, 2000),
                        -rng.uniform(0, 745, 2000), [0.0, -0.0, -1e-300, -744.0, -745.5, -800.0]])
    out = subprocess.run([exe], input="\n".join(float(v).hex() for v in x),
                         capture_output=True, text=True, check=True).stdout.split()
    got = np.array([int(v, 16) for v in out], dtype=np.uint64).view(np.float64)
    lib = oracle_mod.lib()
    ora = np.array([lib.ora_exp_neg(float(v)) for v in x])
    np.testing.assert_array_equal(got, ora)
    ref = np.exp(x)
    normal = ref > 1e-300
    ulp = np.spacing(ref[normal])
    assert np.max(np.abs(got[normal] - ref[normal]) / ulp) <= 1.0
    assert np.all(got[x < -745.2] == 0.0)
