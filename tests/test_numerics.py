"""The oracle's restated third-party numerics against independent references."""
import ctypes
import math

import numpy as np
import pytest

from oracle.runner import build_oracle

FN = ctypes.CFUNCTYPE(ctypes.c_double, ctypes.c_double, ctypes.c_void_p)


@pytest.fixture(scope="module")
def lib():
    L = ctypes.CDLL(build_oracle())
    L.mxo_qag61.argtypes = [FN, ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                            ctypes.c_size_t, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
    L.mxo_r2c_3d.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    L.mxo_c2r_3d.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    return L


@pytest.mark.parametrize("D", [8, 12, 16, 24, 30])
def test_fft_matches_numpy(lib, D):
    rng = np.random.default_rng(D)
    a = rng.standard_normal((D, D, D)).astype(np.float32)
    out = np.zeros((D, D, D // 2 + 1), np.complex64)
    lib.mxo_r2c_3d(D, a.ctypes.data, 0, out.ctypes.data)
    ref = np.fft.rfftn(a.astype(np.float64))
    assert np.abs(out - ref).max() / np.abs(ref).max() < 1e-6
    pad = np.zeros((D, D, 2 * (D // 2 + 1)), np.float32)
    lib.mxo_c2r_3d(D, out.ctypes.data, pad.ctypes.data)
    assert np.abs(pad[:, :, :D] / D ** 3 - a).max() < 1e-5


def _qag(lib, f, a, b, rel, limit=1000):
    res, err = ctypes.c_double(), ctypes.c_double()
    st = lib.mxo_qag61(FN(lambda x, p: f(x)), None, a, b, 0.0, rel, limit, ctypes.byref(res), ctypes.byref(err))
    return st, res.value, err.value


def test_gauss_kronrod_61_is_exact_to_degree_91(lib):
    worst = 0.0
    for k in range(92):
        st, r, _ = _qag(lib, lambda x, k=k: x ** k, -1.0, 1.0, 1e-12, limit=1)
        exact = 2.0 / (k + 1) if k % 2 == 0 else 0.0
        worst = max(worst, abs(r - exact))
    assert worst < 1e-14


def test_qag_adaptive_against_scipy(lib):
    from scipy.integrate import quad

    cases = [(lambda x: math.exp(-x * x), -5.0, 5.0), (lambda x: 1 / math.sqrt(x) if x > 0 else 0.0, 0.0, 1.0),
             (lambda x: math.sin(50 * x) ** 2, 0.0, 3.0), (lambda x: x ** -2.5 * math.exp(-1 / x), 1e-3, 1e3)]
    for f, a, b in cases:
        st, r, _ = _qag(lib, f, a, b, 1e-8)
        ref = quad(f, a, b, epsabs=0, epsrel=1e-11, limit=2000)[0]
        assert abs(r - ref) <= 1e-7 * abs(ref), (r, ref)


def test_natural_spline_against_scipy(lib):
    from scipy.interpolate import CubicSpline

    class Sp(ctypes.Structure):
        _fields_ = [("n", ctypes.c_int), ("x", ctypes.c_void_p), ("y", ctypes.c_void_p), ("c", ctypes.c_void_p)]

    lib.mxo_spline_init.argtypes = [ctypes.POINTER(Sp), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
    lib.mxo_spline_eval.argtypes = [ctypes.POINTER(Sp), ctypes.c_double]
    lib.mxo_spline_eval.restype = ctypes.c_double
    x = np.sort(np.random.default_rng(1).uniform(0, 10, 27))
    y = np.sin(x) * np.exp(-0.1 * x)
    s = Sp()
    lib.mxo_spline_init(ctypes.byref(s), x.ctypes.data, y.ctypes.data, len(x))
    cs = CubicSpline(x, y, bc_type="natural")
    xs = np.linspace(x[0], x[-1], 333)
    got = np.array([lib.mxo_spline_eval(ctypes.byref(s), v) for v in xs])
    assert np.abs(got - cs(xs)).max() < 1e-12
    assert math.isnan(lib.mxo_spline_eval(ctypes.byref(s), x[-1] + 1.0))


def test_brent_bracket(lib):
    class Br(ctypes.Structure):
        _fields_ = [("f", ctypes.c_void_p), ("params", ctypes.c_void_p)] + [
            (n, ctypes.c_double) for n in ("root", "x_lower", "x_upper", "a", "b", "c", "d", "e", "fa", "fb", "fc")]

    f = FN(lambda x, p: math.cos(x) - x)
    lib.mxo_brent_set.argtypes = [ctypes.POINTER(Br), FN, ctypes.c_void_p, ctypes.c_double, ctypes.c_double]
    lib.mxo_brent_iterate.argtypes = [ctypes.POINTER(Br)]
    lib.mxo_root_test_interval.argtypes = [ctypes.c_double] * 4
    b = Br()
    lib.mxo_brent_set(ctypes.byref(b), f, None, 0.0, 1.0)
    for _ in range(100):
        lib.mxo_brent_iterate(ctypes.byref(b))
        if lib.mxo_root_test_interval(b.x_lower, b.x_upper, 0.0, 1e-12) == 0:
            break
    assert abs(b.root - 0.7390851332151607) < 1e-11
