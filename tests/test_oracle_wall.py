"""The wall radiosity exchange in the oracle (Qwall.f90): the boundary-patch
list that MAPB gives (prepare_for_wall_radiation_calculation steps 1-5) is the
one the case builder and reader produce, on every shipped case and on a
synthetic furnace; and one exchange on TC21 case 0041 (gray bands, the wall
sink on) ends converged, with every wall patch in radiative balance."""
import numpy as np
import pytest

from gfm_gb300 import Case, configs
from oracle.pyoracle import Oracle

from .test_case_files import CASES, read_case


def _case_patches(case):
    g = case.grid
    n = g.b_cnt
    cols = [np.ctypeslib.as_array(p, (n,)) for p in (g.b_typ, g.b_i, g.b_j, g.b_k, g.b_orient, g.b_direct)]
    return np.stack(cols, axis=1).astype(np.int32)


@pytest.mark.parametrize("num", CASES)
def test_patch_list_matches_the_mapb_restatement(num, tmp_path):
    case = read_case(num, tmp_path)
    o = Oracle(case)
    assert np.array_equal(o.wall_patch_list(), _case_patches(case))
    o.close()


def test_patch_list_of_the_synthetic_furnace():
    case = Case(configs.small_furnace())
    o = Oracle(case)
    assert np.array_equal(o.wall_patch_list(), _case_patches(case))
    o.wall_setup()   # the flue's exhaust entry covers every exit patch
    o.close()


def test_exchange_converges_with_walls_in_balance(tmp_path):
    case = read_case("0041", tmp_path, kappa=[0.5] * 16, wall_sink=True)
    o = Oracle(case)
    o.initsv()
    o.gflow(3)
    o.wall_setup()
    o.rad_transfer()
    t = o.wall_totals()
    assert t["sweeps"] > 0 and t["outer"] >= 2
    assert t["rel_rad_chg_mean"] < 1e-10
    typ = np.ctypeslib.as_array(case.grid.b_typ, (case.grid.b_cnt,))
    J, qc, qconv, qamb = (o.patch_array(n) for n in ("radiosity", "qc", "q_conv", "q_amb"))
    bt = o.patch_array("b_t")
    # a wall's radiosity is what reaches it minus what it loses (Qwall.f90:1072)
    emis = o.patch_array("emis")
    w = typ == 1
    assert np.all(np.isfinite(bt)) and bt[w].min() >= 200.0
    # its temperature follows from its radiosity (Qwall.f90:1146)
    sig = case.params.sig
    bt_from_j = np.maximum(np.maximum(0.0, (J - (qamb - qconv) * (1 - emis) / emis) / sig) ** 0.25, 200.0)
    # q_conv and q_amb are from the last outer pass, b_T after it: one pass of lag
    assert np.max(np.abs(bt_from_j[w] - bt[w]) / bt[w]) < 1e-6
    # the field carries the wall temperatures at the patch positions
    f = o.download().arrays["t"] * case.params.t0
    bi, bj, bk = (np.ctypeslib.as_array(p, (case.grid.b_cnt,)) for p in (case.grid.b_i, case.grid.b_j, case.grid.b_k))
    assert np.allclose(f[bk[w] - 1, bj[w] - 1, bi[w] - 1], bt[w], rtol=1e-14)
    o.close()
