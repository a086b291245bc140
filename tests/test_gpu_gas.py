"""The band model on the GPU (gas.cu): RAD_GAS and SOOTA of RAD0 in the
volume transfer and in the emission-only source, against the oracle and
against the reference's own radiation record of its converged runs of TC21
case 0041 and the end-fired case 1207 (tests/test_oracle_gas.py)."""
import numpy as np
import pytest

from gfm_gb300 import GpuSolver, abi
from oracle.pyoracle import Oracle

from .test_oracle_gas import RECORD, converged, reference

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("num", ["0041", "1207"])
@pytest.mark.parametrize("prec,tol", [(abi.GFM_PREC_FP64, 1e-9), (abi.GFM_PREC_MIXED, 1e-4)])
def test_transfer_with_band_model_matches_oracle_and_reference(tmp_path, num, prec, tol):
    case, minor = converged(num, tmp_path)
    g = GpuSolver(case, precision=prec)
    g.upload(case.initial_fields())
    g.minor_upload(minor)
    tg = g.rad_transfer()
    o = Oracle(case)
    o.minor_set(minor)
    to = o.rad_transfer()
    ref = reference(num)["rad_detail_last"]
    for mine, theirs in RECORD:
        assert tg[mine] == pytest.approx(to[mine], rel=tol), (mine, tg[mine], to[mine])
        assert tg[mine] == pytest.approx(ref[theirs], rel=tol), (mine, tg[mine], ref[theirs])
    fg, fo = g.download(), o.download()
    for n in ("qa", "qe"):
        assert _rel(fg.arrays[n], fo.arrays[n]) < tol, n
    # the minor species state comes back as it went in
    back = g.minor_download()
    assert back.itr_ms == minor.itr_ms
    assert _rel(back.smf, minor.smf) < (1e-15 if prec == abi.GFM_PREC_FP64 else 1e-7)


@pytest.mark.parametrize("prec,tol", [(abi.GFM_PREC_FP64, 1e-9), (abi.GFM_PREC_MIXED, 1e-4)])
def test_emission_with_band_model_and_soot_gaps_matches_oracle(tmp_path, prec, tol):
    """rad_qe_only with the band model, on a soot field with holes: every
    third cell in loop order without soot, so that SOOTA leaves AKLS as the
    cell before set it (Rad_soot.f90:29) all through the furnace."""
    case, minor = converged("0041", tmp_path)
    lz, nz, mz = case.lp // 2, case.np // 2, case.mp // 2
    k, j, i = np.meshgrid(np.arange(lz), np.arange(nz), np.arange(mz), indexing="ij")
    q = (i * nz + j) * lz + k                       # RAD0's loop order, K fastest
    cells = minor.smf[1::2, 1::2, 1::2]
    cells[q % 3 == 1] = 0.0
    g = GpuSolver(case, precision=prec)
    g.upload(case.initial_fields())
    g.minor_upload(minor)
    g.rad_emission()
    o = Oracle(case)
    o.minor_set(minor)
    o.rad_emission()
    qe_g, qe_o = g.download().arrays["qe"], o.download().arrays["qe"]
    assert np.count_nonzero(qe_o) > 1000
    assert _rel(qe_g, qe_o) < tol


def test_band_model_without_minor_species_is_refused(tmp_path):
    case, _ = converged("0041", tmp_path)
    g = GpuSolver(case)
    g.upload(case.initial_fields())
    with pytest.raises(Exception):
        g.rad_transfer()


def test_wall_exchange_with_band_model_reproduces_melt_handover(tmp_path):
    """The GPU's transfer and wall exchange on the band model, from the
    converged restarts of case 0041: the melt-surface heat flux, the mean
    wall temperature and the heat into the melt against the oracle and
    against the hand-over file the reference's run wrote
    (tests/test_melt_handover.py)."""
    import pathlib
    from gfm_gb300 import logs
    case, minor = converged("0041", tmp_path, wall_sink=True)
    ref = logs.read_melt_flux_file((pathlib.Path(__file__).resolve().parent / "golden" / "case0041" / "logs" /
                                    "it0041m.dat").read_bytes(), case.mp, case.np)
    g = GpuSolver(case, precision=abi.GFM_PREC_FP64)
    g.start()
    g.minor_upload(minor)
    g.wall_setup()
    g.rad_transfer()
    o = Oracle(case)
    o.initsv()
    o.minor_set(minor)
    o.wall_setup()
    o.rad_transfer()
    tg, to = g.wall_totals(), o.wall_totals()
    for k in ("avg_wall_T", "q_melt"):
        assert tg[k] == pytest.approx(to[k], rel=1e-7), k
    assert _rel(g.wall_array("qrs"), o.patch_array("qrs")) < 1e-7
    assert tg["avg_wall_T"] == pytest.approx(ref["avg_wall_T"], rel=1e-6)
    assert tg["q_melt"] == pytest.approx(ref["q_melt"], rel=1e-5)
