"""The oracle iterates the tiny furnace stably, in bounds (checked build)."""
import math

from gfm_gb300 import Case, configs
from oracle.pyoracle import Oracle


def test_oracle_tiny_bounds_checked_through_first_emission_update():
    case = Case(configs.tiny_furnace(nx=9, ny=7, nz=5))
    o = Oracle(case, check_bounds=True)
    o.initsv()
    first, _ = o.gflow(1)
    st, n = o.gflow(59)   # emission-only radiation first runs after iteration 51
    assert n == 59
    assert math.isfinite(st["res_mass"]) and st["res_mass"] < first["res_mass"]
    f = o.download()
    assert f.i1st_rad_qe_done == 1
    assert f.arrays["qe"].max() > 0
