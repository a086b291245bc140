"""Host case construction (GRID3/SETUP/SBC/gen_initial_guess stand-ins)."""
import numpy as np
import pytest

from gfm_gb300 import Case, configs


def propagate_ref(ib_cells: dict, mp, np_, lp):
    """Python restatement of the 27-neighbour face propagation (Grid3.f90:259-275)."""
    ib = np.zeros((lp + 1, np_ + 1, mp + 1), dtype=int)
    for (i, j, k), v in ib_cells.items():
        ib[k, j, i] = v
    ncells = 0
    for i in range(2, mp + 1, 2):
        for j in range(2, np_ + 1, 2):
            for k in range(2, lp + 1, 2):
                b = ib[k, j, i]
                if b <= 0:
                    ncells += 1
                    continue
                for i1 in range(i - 1, i + 2):
                    for j1 in range(j - 1, j + 2):
                        for k1 in range(k - 1, k + 2):
                            if i1 > mp or j1 > np_ or k1 > lp:
                                continue
                            if ib[k1, j1, i1] != 1:
                                ib[k1, j1, i1] = b
    return ib[1:, 1:, 1:], ncells


@pytest.mark.parametrize("mk", [configs.tiny_furnace, lambda: configs.tiny_furnace(nx=9, ny=7, nz=5)])
def test_ibcell_propagation_matches_restatement(mk):
    case = Case(mk())
    ib = case.ibcell()
    cells = {}
    for k in range(2, case.lp + 1, 2):
        for j in range(2, case.np + 1, 2):
            for i in range(2, case.mp + 1, 2):
                cells[(i, j, k)] = int(ib[k - 1, j - 1, i - 1])
    ref, ncells = propagate_ref(cells, case.mp, case.np, case.lp)
    assert np.array_equal(ref, ib)
    assert ncells == case.ncells == mk().ncells_box


def test_small_case_dimensions_and_boundaries():
    cfg = configs.small_furnace()
    case = Case(cfg)
    assert (case.mp, case.np, case.lp) == (100, 52, 36)
    assert case.ncells == 48 * 24 * 16
    ib = case.ibcell()
    cells = ib[1::2, 1::2, 1::2]           # cell centres (even Fortran indices)
    assert set(np.unique(cells)) == {0, 1, 2, 3}
    assert (cells[:, :, 0] >= 1).all() and (cells[:, :, -1] >= 1).all()
    assert (cells[:, :, 0] == 2).sum() > 0 and (cells[:, :, -1] == 3).sum() > 0
    # the pressure reference is an inlet cell, as Sbc.f90:57-63 requires
    g = case.grid
    assert ib[g.k_ref - 1, g.j_ref - 1, g.i_ref - 1] == 2


def test_inlet_mass_flow_consistent():
    case = Case(configs.small_furnace())
    p = case.params
    f = case.initial_fields()
    # gfin0 = (FR_F+FR_OX+FR_N2)/GMFR ~ 1 for inlets without CO2/H2O
    assert f.gfin0 == pytest.approx(1.0, rel=1e-12)
    # reference scales (Setup.f90:542-543, 662-690)
    assert p.ug0 == pytest.approx(p.gmfr / p.dnst0)
    assert p.epsr == pytest.approx(0.05)
    assert p.reyg == pytest.approx(2 * p.dnst0 * p.ug0 / 2.6e-5)
    # fresh start: cell velocities zero, k floor, eps = k^2 (Prop.f90:162-176)
    ib = case.ibcell()
    open_c = (ib[1::2, 1::2, 1::2] == 0)
    k = f.arrays["gf"][3][1::2, 1::2, 1::2][open_c]
    assert np.all(k == 1e-6)
    t = f.arrays["t"][1::2, 1::2, 1::2][open_c] * 500.0
    assert np.all(np.abs(t - 1500.0) <= 15.0 + 1e-9)   # +-1 % seeded noise
    assert t.std() > 1.0


def test_large_case_cells():
    cfg = configs.large_furnace()
    assert cfg.ncells_box == 1179648
