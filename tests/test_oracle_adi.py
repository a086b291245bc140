"""The line solver on manufactured systems: the reference's own solver
self-test recipe (Solvers.f90:1670-1823) -- random off-diagonals, a
diagonally dominant AP, a known solution p(i)=i/2-3 and BS = A p."""
import numpy as np
import pytest

from gfm_gb300 import Case, configs
from oracle.pyoracle import Oracle
from oracle import pyoracle


def manufactured(case, cls=(0, 0, 0), seed=7):
    """A diagonally dominant system on the class `cls` with the known solution
    p = n/2 - 3 (n counting the class's points, the range's border included,
    in K, J, I loop order): AS uniform on [0.1, 1), AP = 1.5 sum AS, BS = A p;
    the start is p on the border and 0 inside."""
    rng = np.random.default_rng(seed)
    shp = (case.lp, case.np, case.mp)
    ap = np.ones(shp)
    as6 = [np.zeros(shp) for _ in range(6)]
    bs = np.zeros(shp)
    ib = case.ibcell()
    mp, np_, lp = case.mp, case.np, case.lp
    ib0, jb0, kb0 = 4 + cls[0], 4 + cls[1], 4 + cls[2]
    ie, je, ke = mp - 2 - cls[0], np_ - 2 - cls[1], lp - 2 - cls[2]
    sol = np.zeros(shp)
    ext = (slice(kb0 - 3, ke + 2, 2), slice(jb0 - 3, je + 2, 2), slice(ib0 - 3, ie + 2, 2))
    nk, nj, ni = [len(range(sl.start, sl.stop, 2)) for sl in ext]
    sol[ext] = (np.arange(nk * nj * ni, dtype=np.float64) / 2.0 - 3.0).reshape(nk, nj, ni)
    inner = (slice(kb0 - 1, ke, 2), slice(jb0 - 1, je, 2), slice(ib0 - 1, ie, 2))
    a = rng.uniform(0.1, 1.0, (nk - 2, nj - 2, ni - 2, 6))
    for q in range(6):
        as6[q][inner] = a[..., q]
    ap[inner] = a.sum(axis=-1) * 1.5
    # BS = AP p - sum AS p_nb, term by term in the order of the offsets below
    offs = [(-2, 0, 0), (2, 0, 0), (0, -2, 0), (0, 2, 0), (0, 0, -2), (0, 0, 2)]
    s = ap[inner] * sol[inner]
    for q, (di, dj, dk) in enumerate(offs):
        nb = (slice(kb0 - 1 + dk, ke + dk, 2), slice(jb0 - 1 + dj, je + dj, 2), slice(ib0 - 1 + di, ie + di, 2))
        s = s - as6[q][inner] * sol[nb]
    bs[inner] = s
    x0 = sol.copy()
    x0[inner] = 0.0  # interior guess 0, boundary = solution
    open_ = np.zeros(shp, bool)
    open_[inner] = True
    open_ &= ib <= 0
    return ap, as6, bs, x0, sol, (ib0, ie, jb0, je, kb0, ke), open_


def test_oracle_adlbl3_converges_to_manufactured_solution():
    case = Case(configs.tiny_furnace())
    ap, as6, bs, x0, sol, rng, open_ = manufactured(case)
    # blocked cells inside the range keep their value: make them exact already
    ib = case.ibcell()
    x0[(ib >= 1)] = sol[(ib >= 1)]
    o = Oracle(case)
    lib = pyoracle.load()
    import ctypes as C
    from gfm_gb300 import abi
    x = x0.copy()
    ptrs = (abi._dp * 6)(*[abi.dptr(a) for a in as6])
    lib.gfo_adlbl3(o.o, abi.dptr(x), abi.dptr(ap), ptrs, abi.dptr(bs), *rng, 200)
    err = np.abs(x - sol)[open_].max()
    assert err < 1e-10, err
    r = lib.gfo_calc_residual(o.o, abi.dptr(x), abi.dptr(ap), ptrs, abi.dptr(bs), *rng)
    assert r < 1e-12


def _oracle_solve(case, sys, nim, adi_mode, rng=None):
    from gfm_gb300 import abi
    ap, as6, bs, x0 = sys[:4]
    o = Oracle(case, adi_mode=adi_mode)
    x = x0.copy()
    ptrs = (abi._dp * 6)(*[abi.dptr(a) for a in as6])
    pyoracle.load().gfo_adlbl3(o.o, abi.dptr(x), abi.dptr(ap), ptrs, abi.dptr(bs), *(rng or sys[5]), nim)
    o.close()
    return x


def test_oracle_redblack_order_converges_and_differs_from_the_march():
    """The red-black plane order (the GPU's production order) solves the same
    system: it converges to the manufactured solution, and after a few sweeps
    its iterate differs from the reference march's, so the order is really
    changed."""
    from gfm_gb300 import abi
    case = Case(configs.tiny_furnace())
    sys = manufactured(case, (0, 1, 0))
    ib = case.ibcell()
    sys[3][ib >= 1] = sys[4][ib >= 1]
    open_ = sys[6]
    x = _oracle_solve(case, sys, 200, abi.GFM_ADI_REDBLACK)
    assert np.abs(x - sys[4])[open_].max() < 1e-10
    xm = _oracle_solve(case, sys, 2, abi.GFM_ADI_MARCH)
    xr = _oracle_solve(case, sys, 2, abi.GFM_ADI_REDBLACK)
    assert np.abs(xm - xr)[open_].max() > 1e-6


def test_oracle_redblack_visit_equals_a_simultaneous_colour_update():
    """One red-black sweep, restated independently in numpy: per half sweep,
    colour 0 planes (IB, IB+4, ..) then colour 1 planes, every plane of a
    colour updated from the same state (ADLZ with L = 1, 2 and the
    averages)."""
    from gfm_gb300 import abi
    case = Case(configs.tiny_furnace())
    ap, as6, bs, x0, sol, rng, open_ = manufactured(case, (0, 0, 0), seed=3)
    ib = case.ibcell()
    got = _oracle_solve(case, (ap, as6, bs, x0, sol, rng), 1, abi.GFM_ADI_REDBLACK)
    ib0, ie, jb, je, kb, ke = rng
    x = x0.copy()

    def line(a_diag, sub, nxt, rhs, x_lo, x_hi, copy, xcur):
        n = len(a_diag)
        pt, qt = np.zeros(n), np.zeros(n)
        p_prev, q_prev = 0.0, x_lo
        for r in range(n):
            alp = a_diag[r] - p_prev * sub[r]
            if abs(alp) <= 1e-20 or copy[r]:
                pt[r], qt[r] = 0.0, xcur[r]
            else:
                pt[r] = nxt[r] / alp
                qt[r] = (rhs[r] + sub[r] * q_prev) / alp
            p_prev, q_prev = pt[r], qt[r]
        out = np.zeros(n)
        v = x_hi
        for r in range(n - 1, -1, -1):
            v = v * pt[r] + qt[r]
            out[r] = v
        return out

    def plane(xs, I):
        i = I - 1
        js = list(range(jb, je + 1, 2))
        ks = list(range(kb, ke + 1, 2))
        for _L in range(2):
            x2, x3 = {}, {}
            for K in ks:
                k = K - 1
                j = np.array(js) - 1
                rhs = bs[k, j, i] + as6[1][k, j, i] * xs[k, j, i + 2] + as6[0][k, j, i] * xs[k, j, i - 2]
                rhs = rhs + as6[5][k, j, i] * xs[k + 2, j, i] + as6[4][k, j, i] * xs[k - 2, j, i]
                r = line(ap[k, j, i], as6[2][k, j, i], as6[3][k, j, i], rhs, xs[k, jb - 3, i], xs[k, je + 1, i],
                         ib[k, j, i] >= 1, xs[k, j, i])
                for J, v in zip(js, r):
                    x2[(J, K)] = v
            for J in js:
                j = J - 1
                k = np.array(ks) - 1
                rhs = bs[k, j, i] + as6[1][k, j, i] * xs[k, j, i + 2] + as6[0][k, j, i] * xs[k, j, i - 2]
                rhs = rhs + as6[3][k, j, i] * xs[k, j + 2, i] + as6[2][k, j, i] * xs[k, j - 2, i]
                r = line(ap[k, j, i], as6[4][k, j, i], as6[5][k, j, i], rhs, xs[kb - 3, j, i], xs[ke + 1, j, i],
                         ib[k, j, i] >= 1, xs[k, j, i])
                for K, v in zip(ks, r):
                    x3[(J, K)] = v
            for (J, K), v in x2.items():
                xs[K - 1, J - 1, i] = (v + x3[(J, K)]) / 2.0

    for _half in range(2):
        for colour in range(2):
            for I in range(ib0 + 2 * colour, ie + 1, 4):
                plane(x, I)
    scale = np.abs(got[open_]).max()
    assert np.abs(got - x)[open_].max() / scale < 1e-13
