"""Known-answer tests pinning the oracle's scalar functions.

The reference ships no tests or golden vectors; these values are derived
independently of the oracle: closed forms of the Fortran formulas, the Planck
integral evaluated by quadrature, and the NIST Shomate expression.
"""
import ctypes as C
import math

import numpy as np
import pytest

from oracle.pyoracle import load


@pytest.fixture(scope="module")
def lib():
    return load()


def test_da_branches(lib):
    # DA(D,F), Prop.f90:97-117: Taylor for Pe<=0.01, |F|/(e^Pe-1) up to 20, 0 above
    assert lib.gfo_da(1e-26, 3.0) == 0.0
    pe = 0.004
    assert lib.gfo_da(1.0, pe) == pytest.approx(1.0 / (1 + pe * (0.5 + pe * (1 / 6 + pe / 24))), rel=1e-15)
    assert lib.gfo_da(2.0, -10.0) == pytest.approx(10.0 / math.expm1(5.0), rel=1e-14)
    assert lib.gfo_da(1.0, 25.0) == 0.0
    # the scheme weight tends to D as Pe -> 0 and is continuous at Pe = 0.01
    assert lib.gfo_da(3.0, 0.0) == 3.0
    a, b = lib.gfo_da(1.0, 0.01), lib.gfo_da(1.0, 0.0100001)
    assert abs(a - b) < 1e-6


def test_tgamf(lib):
    assert lib.gfo_tgamf(11.49) == 1.0
    assert lib.gfo_tgamf(100.0) == pytest.approx(100.0 / (math.log(900.0) * 2.5), rel=1e-15)
    assert lib.gfo_tgamf(11.6) == 1.0  # 11.6/(ln(104.4)*2.5) < 1: clipped to 1
    assert lib.gfo_tgamf(12.0) == pytest.approx(12.0 / (math.log(108.0) * 2.5), rel=1e-15)


def test_emf(lib):
    g1 = (1 - math.exp(-1e-3)) / 1e-3
    assert lib.gfo_emf(0.5, 1e-3) == pytest.approx(5e-4 * g1, rel=1e-15)
    assert lib.gfo_emf(1.0, 2.0) == pytest.approx(1 - math.exp(-2.0), rel=1e-15)


def planck_fraction_above(x: float) -> float:
    """15/pi^4 * integral_x^inf t^3/(e^t-1) dt by quadrature (independent of the series)."""
    from scipy.integrate import quad
    f = lambda t: t ** 3 * math.exp(-t) / -math.expm1(-t)
    val, _ = quad(f, x, x + 200.0, epsabs=1e-15, epsrel=1e-12, limit=400)
    return 15.0 / math.pi ** 4 * val


@pytest.mark.parametrize("x", [0.3, 1.0, 2.5, 4.965, 10.0, 30.0])
def test_rif3_is_planck_fraction(lib, x):
    # RIF(3,0,x), Rad_fun.f90:45-91: fraction of black-body emission with
    # wavelength below hc/(kT x); x = 4.965 is the Wien peak (lambda T = 2898 um K), F = 0.25
    got = lib.gfo_rif3(x)
    assert got == pytest.approx(planck_fraction_above(x), rel=1e-9, abs=1e-15)
    if x == 4.965:
        assert got == pytest.approx(0.25, abs=1e-3)


def test_zy1_table_lookup(lib):
    xs = np.array([1.0, 2.0, 4.0])
    ys = np.array([10.0, 20.0, 0.0])
    dp = C.POINTER(C.c_double)
    f = lambda v: lib.gfo_zy1(xs.ctypes.data_as(dp), ys.ctypes.data_as(dp), v, 3)
    assert f(0.5) == 5.0         # below the table: proportional
    assert f(1.5) == 15.0        # linear inside
    assert f(3.0) == 10.0
    assert f(9.0) == 0.0         # beyond: last value


def _y9(**kw):
    y = np.zeros(9)
    idx = {"yf": 0, "yo2": 1, "h": 2, "k": 3, "eps": 4, "yco2": 5, "yn2": 6, "yh2o": 8}
    for k, v in kw.items():
        y[idx[k]] = v
    return y


def test_shomate_quirk_pure_nitrogen(lib):
    # T_to_enth, Prop.f90:537-562, pure N2 at 1000 K.  The reference accumulates
    # f_mix = d_mix + Y*F and h_mix = e_mix + Y*H inside the species loop, so for
    # a mixture without H2O (last species) F and H drop out: f_mix = d_mix,
    # h_mix = e_mix.  NIST's own value would be 21.46 kJ/mol; the reference gives
    # A t + B/2 t^2 + C/3 t^3 + D/4 t^4 - E/t + D - E.
    A, B, Cc, D, E = 26.092, 8.218801, -1.976141, 0.159274, 0.044434
    t = 1.0
    kj_mol = t * (A + t * (B / 2 + t * (Cc / 3 + t * (D / 4)))) - E / t + D - E
    h0 = 1.0057e3 * (5.0e2 - 298.15)
    expected = kj_mol * 1e6 / (28.0134 * h0)
    y = _y9(yn2=1.0)
    dp = C.POINTER(C.c_double)
    got = lib.gfo_t_to_enth(y.ctypes.data_as(dp), 1000.0 / 500.0)
    assert got == pytest.approx(expected, rel=1e-13)
    # the quirk is real: this is far from the textbook 21.46 kJ/mol
    assert kj_mol == pytest.approx(29.65, abs=0.01)


@pytest.mark.parametrize("T", [350.0, 900.0, 1250.0, 1650.0, 2400.0])
def test_enth_temperature_round_trip(lib, T):
    # enth_to_T inverts T_to_enth when Newton starts from the cell's previous
    # temperature, as GFLOW does (Gflow.f90:311; Prop.f90:434)
    y = _y9(yf=0.05, yo2=0.1, yco2=0.12, yn2=0.6, yh2o=0.13)
    dp = C.POINTER(C.c_double)
    h = lib.gfo_t_to_enth(y.ctypes.data_as(dp), T / 500.0)
    back = lib.gfo_enth_to_t(y.ctypes.data_as(dp), h, T / 500.0 * (1 + 1e-3))
    assert back * 500.0 == pytest.approx(T, abs=1e-6)


def test_enth_to_t_depends_on_newton_start_across_set_switches(lib):
    # Switching a species between its low/high Shomate sets inside the Newton
    # loop rewrites f_mix/h_mix from the last switched species only
    # (Prop.f90:456-495), so the root found depends on the starting guess when
    # the path crosses a cut-off temperature.  The oracle keeps this behaviour.
    y = _y9(yf=0.05, yo2=0.1, yco2=0.12, yn2=0.6, yh2o=0.13)
    dp = C.POINTER(C.c_double)
    h = lib.gfo_t_to_enth(y.ctypes.data_as(dp), 1250.0 / 500.0)
    near = lib.gfo_enth_to_t(y.ctypes.data_as(dp), h, 1250.0 / 500.0) * 500.0
    far = lib.gfo_enth_to_t(y.ctypes.data_as(dp), h, 1500.0 / 500.0) * 500.0
    assert near == pytest.approx(1250.0, abs=1e-6)
    assert abs(far - 1250.0) > 10.0


def test_conc_closure(lib):
    dp = C.POINTER(C.c_double)
    y = _y9(yf=0.1, yo2=0.2, yco2=0.1, yn2=0.5)
    lib.gfo_conc(y.ctypes.data_as(dp))
    assert y[8] == pytest.approx(0.1, abs=1e-15)  # H2O = 1 - sum
    y = _y9(yf=0.5, yo2=0.4, yco2=0.2, yn2=0.3, yh2o=0.1)
    lib.gfo_conc(y.ctypes.data_as(dp))
    s = y[0] + y[1] + y[5] + y[6] + y[8]
    assert s == pytest.approx(1.0, abs=1e-15)   # over-full mixture renormalised
