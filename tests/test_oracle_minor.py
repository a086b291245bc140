"""The minor species and soot of MSFLOW in the oracle (Msflow.f90, Gslv3m.f90,
Sourcem.f90, with INITSVM, EXTRM, INTPM), checked against the reference's own
converged run of TC21 case 0041.

The reference ends a run with SAV3F (rg0041c.d), INITSVM from the previous
minor species restart, MSFLOW of 300 iterations on the final flow, and SAV3FM
(rs0041c.d) (A0main.f90:205-223).  The state it stored is therefore what 300
MSFLOW iterations make of the state before, on that flow; after 129 such
calls it is close to MSFLOW's fixed point on it.  300 more iterations of the
oracle's MSFLOW from it, on the flow of rg0041c.d, have to stay close to it:
the reference's own MSFLOW does not settle below residuals of about 1e-4
(CH4) to 1e-13 (H2O) (its mresid logs), so the bound is a few parts per
thousand, not the FP64 level; a wrong rate, sign or unit moves the species
by tens of percent within tens of iterations."""
import numpy as np
import pytest

from gfm_gb300 import abi
from oracle.pyoracle import Oracle

from .test_oracle_gas import converged

NAMES = ("CH4", "O2", "CO", "H2O", "CO2", "N2", "NO")


def _rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def test_msflow_stays_at_the_reference_converged_state(tmp_path):
    case, minor = converged("0041", tmp_path)
    o = Oracle(case)
    o.initsv()
    o.gflow(1)   # GSLV3G leaves its coefficients for GSLV3M's first reaction pass
    o.minor_set(minor)
    o.initsvm(restart=True)
    st = o.msflow(300)
    assert st["itr_ms"] == minor.itr_ms + 300 and st["iterations"] == 300 and st["converged"] == 0
    got = o.minor_get()
    s = (slice(1, None, 2),) * 3
    open_ = case.ibcell()[s] <= 0
    bound = {"CH4": 1e-2, "O2": 2e-2, "CO": 3e-2, "H2O": 1e-2, "CO2": 1e-2, "N2": 1e-3, "NO": 5e-3}
    for l, n in enumerate(NAMES):
        err = _rel_l2(got.gfm[l][s][open_], minor.gfm[l][s][open_])
        assert err < bound[n], (n, err)
    assert _rel_l2(got.smf[s][open_], minor.smf[s][open_]) < 6e-2
    # the residual levels of the reference's own MSFLOW
    r = st["resid_ms"]
    assert r[0] < 1e-4 and r[1] < 1e-5 and max(r[2:7]) < 1e-8
    # fuel burns as fast as it comes in; soot stays under its cap
    assert got.rrms[0].sum() == pytest.approx(case.summary["fr_f"] / 16.0426, rel=0.1)
    assert 0 < st["smf_max"] <= case.params.soot_cap and st["soot_tot"] > 0
    assert 0 < st["svf_r"] < 1e-6 and 0 < st["bal_ms"] < 0.1


def test_initsvm_new_start(tmp_path):
    case, _ = converged("0041", tmp_path)
    o = Oracle(case)
    o.initsv()
    o.initsvm(restart=False)
    m = o.minor_get()
    gf = o.download().arrays["gf"]
    s = (slice(1, None, 2),) * 3
    for l, gl in ((0, 0), (1, 1), (3, 8), (4, 5), (5, 6)):
        assert np.array_equal(m.gfm[l][s], gf[gl][s])
    assert not m.gfm[2].any() and not m.gfm[6].any() and not m.smf.any()
    # INTPM fills the faces between open cells
    ib = case.ibcell()
    zf = (slice(2, -1, 2), slice(1, None, 2), slice(1, None, 2))   # K odd, J and I even
    inner = ib[zf] == 0
    assert np.all(m.gfm[5][zf][inner] > 0)


def test_first_emission_update_runs_msflow(tmp_path):
    """SPHASE's first emission update after iteration 50 runs INITSVM (a
    restart: IRSTYPM = 1 and a state is there) and MSFLOW(300) first
    (Sphase.f90:210-224), then the emission on the band model."""
    case, minor = converged("0041", tmp_path, rad_emission=True)
    f = case.initial_fields()
    f.i1st_rad_qe_done = 0
    f.do_rad_qe_only_cnt = 9
    o = Oracle(case, fields=f)
    o.initsv()
    o.minor_set(minor)
    o.gflow(1)
    m = o.minor_get()
    assert m.itr_ms == minor.itr_ms + 300
    assert o.download().i1st_rad_qe_done == 1
    assert np.count_nonzero(o.download().arrays["qe"]) > 1000
