"""MSFLOW on the GPU (minor.cu, INITSVM/EXTRM/INTPM in bc.cu) against the
oracle's restatement, from the reference's converged TC21 case 0041 (its gas
and minor species restarts): the seven species, soot, the reaction rates and
MSFLOW's report; and SPHASE's first emission update, which runs INITSVM and
MSFLOW(300) before the band-model emission.

MSFLOW is chaotic on this case: last-bit differences between the GPU and the
oracle grow about tenfold every five iterations (1e-16 after two, 1e-12
after 20, 1e-9 after 40) and stop at about 1e-2 from iteration 80 on, the
size of MSFLOW's own oscillation (the reference's minor species residuals
level off, they do not fall).  So the arithmetic is pinned through 20
iterations in FP64, and longer runs are held to that oscillation's size."""
import numpy as np
import pytest

from gfm_gb300 import GpuSolver, abi
from oracle.pyoracle import Oracle

from .test_oracle_gas import converged

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _pair(tmp_path, prec, adi, **kw):
    case, minor = converged("0041", tmp_path, **kw)
    g = GpuSolver(case, adi_mode=adi, precision=prec)
    g.start()
    o = Oracle(case, adi_mode=adi)
    o.initsv()
    return case, minor, g, o


def _compare_minor(mg, mo, tol, rrms_tol):
    for l in range(7):
        assert _rel(mg.gfm[l], mo.gfm[l]) < tol, ("gfm", l)
    assert _rel(mg.smf, mo.smf) < tol
    assert _rel(mg.bs_soot_prev, mo.bs_soot_prev) < tol and _rel(mg.sfp_soot_prev, mo.sfp_soot_prev) < tol
    for q in (0, 1, 3):
        assert _rel(mg.rrms[q], mo.rrms[q]) < rrms_tol, ("rrms", q)


@pytest.mark.parametrize("prec,adi,n,tol,rtol", [
    (abi.GFM_PREC_FP64, abi.GFM_ADI_MARCH, 5, 1e-9, 1e-9),
    (abi.GFM_PREC_FP64, abi.GFM_ADI_REDBLACK, 20, 1e-9, 1e-9),
    (abi.GFM_PREC_MIXED, abi.GFM_ADI_REDBLACK, 5, 1e-4, 1e-3),
    (abi.GFM_PREC_FP64, abi.GFM_ADI_REDBLACK, 300, 5e-2, 1e-1),
])
def test_msflow_matches_oracle(tmp_path, prec, adi, n, tol, rtol):
    case, minor, g, o = _pair(tmp_path, prec, adi)
    g.gflow(1)
    o.gflow(1)
    g.minor_upload(minor)
    o.minor_set(minor)
    g.initsvm(restart=True)
    o.initsvm(restart=True)
    sg, so = g.msflow(n), o.msflow(n)
    assert sg["itr_ms"] == so["itr_ms"] == minor.itr_ms + n
    _compare_minor(g.minor_download(), o.minor_get(), tol, rtol)
    for k in ("bal_ms", "soot_tot", "smf_max", "smf_max_noclip", "svf_r"):
        assert sg[k] == pytest.approx(so[k], rel=max(tol, 1e-12)), k
    for l in range(7):
        assert sg["gfm_out"][l] == pytest.approx(so["gfm_out"][l], rel=max(tol, 1e-12), abs=1e-18), l
    if prec == abi.GFM_PREC_FP64 and n <= 20:
        for l in range(8):
            assert sg["resid_ms"][l] == pytest.approx(so["resid_ms"][l], rel=1e-6), l


def test_initsvm_new_start_matches_oracle(tmp_path):
    case, _, g, o = _pair(tmp_path, abi.GFM_PREC_FP64, abi.GFM_ADI_REDBLACK)
    g.initsvm(restart=False)
    o.initsvm(restart=False)
    mg, mo = g.minor_download(), o.minor_get()
    for l in range(7):
        assert _rel(mg.gfm[l], mo.gfm[l]) < 1e-13, l
    assert not mg.smf.any()


def test_first_emission_update_runs_msflow(tmp_path):
    case, minor = converged("0041", tmp_path, rad_emission=True)
    g = GpuSolver(case, adi_mode=abi.GFM_ADI_MARCH, precision=abi.GFM_PREC_FP64)
    g.upload(_with_trigger(case))
    g.initsv()
    o = Oracle(case, fields=_with_trigger(case), adi_mode=abi.GFM_ADI_MARCH)
    o.initsv()
    g.minor_upload(minor)
    o.minor_set(minor)
    g.gflow(1)
    o.gflow(1)
    mg, mo = g.minor_download(), o.minor_get()
    assert mg.itr_ms == mo.itr_ms == minor.itr_ms + 300
    _compare_minor(mg, mo, 5e-2, 1e-1)   # 300 MSFLOW iterations: the oscillation's size
    fg, fo = g.download(), o.download()
    assert fg.i1st_rad_qe_done == fo.i1st_rad_qe_done == 1
    assert _rel(fg.arrays["qe"], fo.arrays["qe"]) < 1e-2


def _with_trigger(case):
    f = case.initial_fields()
    f.i1st_rad_qe_done = 0
    f.do_rad_qe_only_cnt = 9
    return f
