"""The oracle's own start-up of the synthetic furnace (gfo_case_build) against
the product's (gfm_case_build): the same grid, cell map, constants, wall
patches, kinetics table and fresh-start fields.  The two are written
independently (the oracle's from the Fortran start-up routines, GRID3, SETUP,
SBC and gen_initial_guess), so agreement pins the product's builder; the
oracle's start-up is what the benchmark's reference arm runs from."""
import numpy as np
import pytest

from gfm_gb300 import Case, configs
from oracle.pyoracle import Oracle, OracleCase

CFGS = [configs.tiny_furnace(), configs.small_furnace(), configs.furnace_variant(3, 40, 20, 14, aspect=2.5),
        configs.large_furnace(seed=12)]


def _arr(ptr, n):
    return np.ctypeslib.as_array(ptr, shape=(n,)).copy()


@pytest.mark.parametrize("cfg", CFGS, ids=[c.name for c in CFGS])
def test_oracle_start_up_matches_the_product_builder(cfg):
    a, b = Case(cfg), OracleCase(cfg)
    ga, gb = a.grid, b.grid
    assert (ga.mp, ga.np, ga.lp, ga.ncells) == (gb.mp, gb.np, gb.lp, gb.ncells)
    assert (ga.i_ref, ga.j_ref, ga.k_ref, ga.p_ref) == (gb.i_ref, gb.j_ref, gb.k_ref, gb.p_ref)
    for name, n in (("x", ga.mp), ("dx", ga.mp), ("r", ga.np), ("dr", ga.np), ("rs", ga.np), ("z", ga.lp),
                    ("dz", ga.lp)):
        assert np.array_equal(_arr(getattr(ga, name), n), _arr(getattr(gb, name), n)), name
    assert np.array_equal(a.ibcell(), b.ibcell())
    assert ga.b_cnt == gb.b_cnt
    for name in ("b_typ", "b_i", "b_j", "b_k", "b_orient", "b_direct", "b_t"):
        assert np.array_equal(_arr(getattr(ga, name), ga.b_cnt), _arr(getattr(gb, name), gb.b_cnt)), name
    assert ga.nr0 == gb.nr0 and ga.nwl == gb.nwl
    for name in ("rtim", "delrt", "hrt", "delr", "timed", "hrd"):
        assert np.array_equal(_arr(getattr(ga, name), ga.nr0), _arr(getattr(gb, name), gb.nr0)), name
    for name in ("wl", "akl0"):
        assert np.array_equal(_arr(getattr(ga, name), ga.nwl), _arr(getattr(gb, name), gb.nwl)), name
    pa, pb = a.params, b.params
    for f, _ in pa._fields_:
        va, vb = getattr(pa, f), getattr(pb, f)
        if hasattr(va, "__len__"):
            assert list(va) == list(vb), f
        else:
            assert va == vb, f
    fa, fb = a.initial_fields(), b.initial_fields()
    for k in fa.arrays:
        x, y = fa.arrays[k], fb.arrays[k]
        scale = max(np.abs(x).max(), 1e-300)
        assert np.abs(x - y).max() <= 1e-15 * scale, (k, np.abs(x - y).max() / scale)
    assert (fa.gfin0, fa.q_h_in, fa.factor) == pytest.approx((fb.gfin0, fb.q_h_in, fb.factor), rel=1e-15)


def test_oracle_runs_from_its_own_start_up():
    """An oracle iteration from the oracle's start-up is the iteration from
    the product's start-up (the reference arm of the benchmark runs the
    former)."""
    cfg = configs.tiny_furnace()
    outs = []
    for case in (Case(cfg), OracleCase(cfg)):
        o = Oracle(case)
        o.initsv()
        st, _ = o.gflow(3)
        outs.append((st, o.download()))
        o.close()
    (sa, fa), (sb, fb) = outs
    assert sa["res_mass"] == pytest.approx(sb["res_mass"], rel=1e-12)
    for k in ("p", "t", "ug"):
        assert np.allclose(fa.arrays[k], fb.arrays[k], rtol=1e-11, atol=1e-14), k


def test_oracle_half_blocked_factors_take_effect(tmp_path):
    """The oracle's VOL_C0 and AREA_C scale by BV_F and BA_F: one iteration
    of TC21 case 0041 with half-blocked cells moves with the factors, and
    stays finite."""
    import shutil
    from gfm_gb300 import Case
    from .test_case_files import GOLD, INPUTS, half_blocked_dir
    src = tmp_path / "src"
    src.mkdir()
    for n in INPUTS:
        shutil.copyfile(GOLD / n, src / n)
    d = half_blocked_dir(src, tmp_path / "half")
    ones = tmp_path / "ones"
    ones.mkdir()
    for n in INPUTS:
        shutil.copyfile(d / n, ones / n)
    gd = (ones / "gd0041c.dat").read_text()
    start = gd.index("&GRD")
    (ones / "gd0041c.dat").write_text(gd[:start] + "&GRD\n/\n")
    res = []
    for dd in (d, ones):
        o = Oracle(Case.from_files(dd, "0041"))
        o.initsv()
        st = o.gflow(1)[0]
        f = o.download()
        o.close()
        assert np.all(np.isfinite(f.arrays["p"])) and np.all(np.isfinite(f.arrays["t"]))
        res.append((st["res_mass"], f.arrays["p"].copy()))
    assert res[0][0] != res[1][0]
    assert not np.array_equal(res[0][1], res[1][1])
