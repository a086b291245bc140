"""Line solver through gfm_gpu_adlbl3 on manufactured systems
(the reference's solver self-test recipe, Solvers.f90:1670-1823)."""
import ctypes as C

import numpy as np
import pytest

from gfm_gb300 import Case, GpuSolver, abi, configs
from oracle import pyoracle
from oracle.pyoracle import Oracle
from tests.test_oracle_adi import manufactured

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("cls", [(0, 0, 0), (1, 0, 0), (0, 1, 0)])
def test_march_matches_oracle_adlbl3(cls):
    case = Case(configs.small_furnace())
    ap, as6, bs, x0, sol, rng, open_ = manufactured(case, cls)
    g = GpuSolver(case, adi_mode=abi.GFM_ADI_MARCH)
    xg = g.adlbl3(x0, ap, as6, bs, *rng, 2)
    o = Oracle(case)
    lib = pyoracle.load()
    xo = x0.copy()
    ptrs = (abi._dp * 6)(*[abi.dptr(a) for a in as6])
    lib.gfo_adlbl3(o.o, abi.dptr(xo), abi.dptr(ap), ptrs, abi.dptr(bs), *rng, 2)
    err = np.abs(xg - xo)[open_].max() / np.abs(xo[open_]).max()
    assert err < 1e-13, err
    g.close()


@pytest.mark.parametrize("prec,tol", [(abi.GFM_PREC_FP64, 1e-10), (abi.GFM_PREC_MIXED, 1e-4)])
def test_redblack_converges_to_manufactured_solution(prec, tol):
    case = Case(configs.small_furnace())
    ap, as6, bs, x0, sol, rng, open_ = manufactured(case)
    ib = case.ibcell()
    x0[ib >= 1] = sol[ib >= 1]
    g = GpuSolver(case, adi_mode=abi.GFM_ADI_REDBLACK, precision=prec)
    x = g.adlbl3(x0, ap, as6, bs, *rng, 100)
    err = np.abs(x - sol)[open_].max() / np.abs(sol[open_]).max()
    assert err < tol, err
    g.close()


def _oracle_adlbl3(case, adi, ap, as6, bs, x0, rng, nim):
    o = Oracle(case, adi_mode=adi)
    xo = x0.copy()
    ptrs = (abi._dp * 6)(*[abi.dptr(a) for a in as6])
    pyoracle.load().gfo_adlbl3(o.o, abi.dptr(xo), abi.dptr(ap), ptrs, abi.dptr(bs), *rng, nim)
    o.close()
    return xo


@pytest.mark.parametrize("plane", ["1", "0"])
@pytest.mark.parametrize("cls", [(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1)])
@pytest.mark.parametrize("prec,tol", [(abi.GFM_PREC_FP64, 1e-13), (abi.GFM_PREC_MIXED, 1e-5)])
def test_redblack_matches_the_redblack_oracle(cls, prec, tol, plane, monkeypatch):
    """Two sweeps in the red-black plane order against the oracle's ADLBL3 in
    the same order, on each face class: the same iterate up to rounding
    (FP64) or to FP32 rounding (mixed).  Both forms of the order: one CTA per
    plane visit (default), and the segmented colour passes (GFM_RB_PLANE=0,
    read when the handle is created)."""
    monkeypatch.setenv("GFM_RB_PLANE", plane)
    case = Case(configs.small_furnace())
    ap, as6, bs, x0, sol, rng, open_ = manufactured(case, cls)
    g = GpuSolver(case, adi_mode=abi.GFM_ADI_REDBLACK, precision=prec)
    xg = g.adlbl3(x0, ap, as6, bs, *rng, 2)
    g.close()
    xo = _oracle_adlbl3(case, abi.GFM_ADI_REDBLACK, ap, as6, bs, x0, rng, 2)
    err = np.abs(xg - xo)[open_].max() / np.abs(xo[open_]).max()
    assert err < tol, err


@pytest.mark.parametrize("prec,tol", [(abi.GFM_PREC_FP64, 1e-13), (abi.GFM_PREC_MIXED, 1e-5)])
def test_redblack_large_planes_match_the_redblack_oracle(prec, tol):
    """The 192x96x64 furnace's planes (96 x 64 points) take the plane visit on
    CTAs of 768 threads (the smaller cases above fit the 256-thread form):
    one sweep against the oracle in the same plane order."""
    case = Case(configs.large_furnace())
    ap, as6, bs, x0, sol, rng, open_ = manufactured(case, (0, 0, 1))
    g = GpuSolver(case, adi_mode=abi.GFM_ADI_REDBLACK, precision=prec)
    xg = g.adlbl3(x0, ap, as6, bs, *rng, 1)
    g.close()
    xo = _oracle_adlbl3(case, abi.GFM_ADI_REDBLACK, ap, as6, bs, x0, rng, 1)
    err = np.abs(xg - xo)[open_].max() / np.abs(xo[open_]).max()
    assert err < tol, err


@pytest.mark.parametrize("adi,plane", [(abi.GFM_ADI_MARCH, "1"), (abi.GFM_ADI_REDBLACK, "1"),
                                       (abi.GFM_ADI_REDBLACK, "0")])
def test_single_z_row_takes_the_y_pass_alone(adi, plane, monkeypatch):
    """A solve range with one z-row (kb == ke): the reference's ADLZ copies the
    first y-line pass into XT and leaves the plane (Adlbl3.f90:124-130)."""
    monkeypatch.setenv("GFM_RB_PLANE", plane)
    case = Case(configs.small_furnace())
    ap, as6, bs, x0, sol, rng, open_ = manufactured(case)
    ib0, ie, jb, je, kb, ke = rng
    one = (ib0, ie, jb, je, kb + 6, kb + 6)
    g = GpuSolver(case, adi_mode=adi)
    xg = g.adlbl3(x0, ap, as6, bs, *one, 2)
    g.close()
    xo = _oracle_adlbl3(case, adi, ap, as6, bs, x0, one, 2)
    sel = np.zeros_like(open_)
    sel[kb + 5, jb - 1:je:2, ib0 - 1:ie:2] = True
    sel &= open_
    assert np.abs(xg - xo)[sel].max() / np.abs(xo[sel]).max() < 1e-13
    assert np.array_equal(xg[~sel], x0[~sel])


@pytest.mark.parametrize("prec", [abi.GFM_PREC_FP64, abi.GFM_PREC_MIXED])
@pytest.mark.parametrize("cls", [(0, 0, 0), (0, 1, 1)])
def test_redblack_launch_forms_agree_bit_for_bit(prec, cls, monkeypatch):
    """Segmented colour passes (GFM_RB_PLANE=0): pass L=2 averaging the pass
    L=1 results where it reads them (default) and the separate averaging
    launch compute the same values in the same order, with and without
    programmatic dependent launch: identical iterates."""
    monkeypatch.setenv("GFM_RB_PLANE", "0")
    case = Case(configs.small_furnace())
    ap, as6, bs, x0, sol, rng, open_ = manufactured(case, cls)
    out = []
    for avg, pdl in (("1", "1"), ("0", "1"), ("1", "0"), ("0", "0")):
        monkeypatch.setenv("GFM_RB_AVG_IN_PASS", avg)
        monkeypatch.setenv("GFM_PDL", pdl)
        g = GpuSolver(case, adi_mode=abi.GFM_ADI_REDBLACK, precision=prec)
        out.append(g.adlbl3(x0, ap, as6, bs, *rng, 5))
        g.close()
    for o in out[1:]:
        assert np.array_equal(o, out[0])


@pytest.mark.parametrize("prec", [abi.GFM_PREC_FP64, abi.GFM_PREC_MIXED])
def test_plane_visit_with_and_without_dependent_launch(prec, monkeypatch):
    """The plane-visit form gives identical iterates with and without
    programmatic dependent launch of its kernels."""
    monkeypatch.setenv("GFM_RB_PLANE", "1")
    case = Case(configs.small_furnace())
    ap, as6, bs, x0, sol, rng, open_ = manufactured(case, (0, 1, 1))
    out = []
    for pdl in ("1", "0"):
        monkeypatch.setenv("GFM_PDL", pdl)
        g = GpuSolver(case, adi_mode=abi.GFM_ADI_REDBLACK, precision=prec)
        out.append(g.adlbl3(x0, ap, as6, bs, *rng, 5))
        g.close()
    assert np.array_equal(out[0], out[1])
