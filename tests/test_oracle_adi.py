"""The line solver on manufactured systems: the reference's own solver
self-test recipe (Solvers.f90:1670-1823) -- random off-diagonals, a
diagonally dominant AP, a known solution p(i)=i/2-3 and BS = A p."""
import numpy as np
import pytest

from gfm_gb300 import Case, configs
from oracle.pyoracle import Oracle
from oracle import pyoracle


def manufactured(case, cls=(0, 0, 0), seed=7):
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
    n = 0
    for k in range(kb0 - 2, ke + 3, 2):
        for j in range(jb0 - 2, je + 3, 2):
            for i in range(ib0 - 2, ie + 3, 2):
                sol[k - 1, j - 1, i - 1] = n / 2.0 - 3.0
                n += 1
    for k in range(kb0, ke + 1, 2):
        for j in range(jb0, je + 1, 2):
            for i in range(ib0, ie + 1, 2):
                a = rng.uniform(0.1, 1.0, 6)
                for q in range(6):
                    as6[q][k - 1, j - 1, i - 1] = a[q]
                ap[k - 1, j - 1, i - 1] = a.sum() * 1.5
    # BS = AP p - sum AS p_nb over open cells; blocked cells keep their value
    offs = [(-2, 0, 0), (2, 0, 0), (0, -2, 0), (0, 2, 0), (0, 0, -2), (0, 0, 2)]
    for k in range(kb0, ke + 1, 2):
        for j in range(jb0, je + 1, 2):
            for i in range(ib0, ie + 1, 2):
                s = ap[k - 1, j - 1, i - 1] * sol[k - 1, j - 1, i - 1]
                for q, (di, dj, dk) in enumerate(offs):
                    s -= as6[q][k - 1, j - 1, i - 1] * sol[k - 1 + dk, j - 1 + dj, i - 1 + di]
                bs[k - 1, j - 1, i - 1] = s
    x0 = sol.copy()
    x0[kb0 - 1:ke:2, jb0 - 1:je:2, ib0 - 1:ie:2] = 0.0  # interior guess 0, boundary = solution
    open_ = np.zeros(shp, bool)
    open_[kb0 - 1:ke:2, jb0 - 1:je:2, ib0 - 1:ie:2] = True
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
