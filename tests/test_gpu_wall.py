"""The wall radiosity exchange on the GPU (gfm_gpu_wall_setup, the end of
gfm_gpu_rad_transfer) against the oracle's restatement of wallq: TC21 case
0041 read from its files with gray bands and the wall sink.  The GPU sweeps
read the previous sweep's radiosities where the reference (and the oracle)
update in patch order; both stop on the reference's rules (mean relative
change below 1e-10), so the patch temperatures and radiosities agree to the
distance of the two stopping points from the common fixed point, and the
iterations after the exchange carry it."""
import numpy as np
import pytest

from gfm_gb300 import GpuSolver, abi
from oracle.pyoracle import Oracle

from .test_case_files import read_case
from .test_gpu_parity import field_errors

pytestmark = pytest.mark.gpu

ARRAYS = ("b_t", "radiosity", "q_amb", "q_conv", "qc", "qeb", "emis", "b_face_area", "patch_area")


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


# FP64: three iterations before the exchange and two after; mixed: one and
# one, since this case's velocities in FP32 leave 1e-4 after a few
# iterations whatever the radiation (test_gpu_case_files)
@pytest.mark.parametrize("prec,adi,tol_wall,tol_field,n0,n1", [
    (abi.GFM_PREC_FP64, abi.GFM_ADI_MARCH, 1e-7, 1e-6, 3, 2),
    (abi.GFM_PREC_FP64, abi.GFM_ADI_REDBLACK, 1e-7, 1e-6, 3, 2),
    (abi.GFM_PREC_MIXED, abi.GFM_ADI_REDBLACK, 1e-4, 1e-4, 1, 1),
])
def test_exchange_matches_oracle(tmp_path, prec, adi, tol_wall, tol_field, n0, n1):
    case = read_case("0041", tmp_path, kappa=[0.5] * 16, wall_sink=True)
    g = GpuSolver(case, adi_mode=adi, precision=prec)
    g.start()
    o = Oracle(case, adi_mode=adi)
    o.initsv()
    g.gflow(n0)
    o.gflow(n0)
    g.wall_setup()
    o.wall_setup()
    g.rad_transfer()
    o.rad_transfer()
    tg, to = g.wall_totals(), o.wall_totals()
    assert tg["b_cnt"] == to["b_cnt"] and tg["rel_rad_chg_mean"] < 1e-10
    msg = {k: (tg[k], to[k]) for k in ("sweeps", "outer", "avg_wall_T", "q_melt", "q_wall_loss")}
    for n in ARRAYS:
        assert _rel(g.wall_array(n), o.patch_array(n)) < tol_wall, (n, msg)
    for k in ("avg_wall_T", "q_melt", "q_wall_loss", "q_incident_total", "q_rad_inlet", "q_rad_outlet"):
        assert tg[k] == pytest.approx(to[k], rel=tol_wall, abs=1e-6), (k, msg)
    # the field after the exchange (wall T at the patches) and two more iterations
    err = field_errors(g.download(), o.download(), case.ibcell() <= 0)
    assert max(err.values()) < tol_field, err
    g.gflow(n1)
    o.gflow(n1)
    err = field_errors(g.download(), o.download(), case.ibcell() <= 0)
    assert max(err.values()) < 10 * tol_field, err
    g.close()
    o.close()


def test_second_exchange_continues_from_the_first(tmp_path):
    """Later calls keep the wall temperatures (only melt patches are reset,
    Rad_emis.f90:260-273) and converge again."""
    case = read_case("0041", tmp_path, kappa=[0.5] * 16, wall_sink=True)
    g = GpuSolver(case, adi_mode=abi.GFM_ADI_REDBLACK, precision=abi.GFM_PREC_FP64)
    g.start()
    g.gflow(2)
    g.wall_setup()
    g.rad_transfer()
    t1 = g.wall_totals()
    g.gflow(2)
    g.rad_transfer()
    t2 = g.wall_totals()
    assert t2["sweeps"] > t1["sweeps"] and t2["rel_rad_chg_mean"] < 1e-10
    assert abs(t2["avg_wall_T"] - t1["avg_wall_T"]) < 0.05 * t1["avg_wall_T"]
    g.close()
