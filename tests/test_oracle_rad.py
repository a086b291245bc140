"""Volume radiation transfer in the CPU oracle (RAD0 + QRNF/QREF/QRTX/Y/Z,
combustion/Code/Qrn.f90, Qre.f90, Qrt[xyz].f90): the angle function against
libm, conservation of the traced energy, and the emission total against
RAD0's band total.  The reference has no radiation tests or golden vectors;
these are the properties its own diagnostics print (Qrn.f90:190-208: q_diff
is emission minus everything absorbed or deposited)."""
import math

import numpy as np
import pytest

from gfm_gb300 import Case, configs
from oracle.pyoracle import Oracle, load


@pytest.mark.parametrize("x", [0.0, 1e-12, 1e-3, 0.1, 0.26794919243112270647, 0.2679492, 0.5, 0.99999, 1.0,
                               1.00001, 2.0, 7.5, 1e3, 1e12])
def test_atand_matches_libm(x):
    lib = load()
    want = math.degrees(math.atan(x))
    got = lib.gfo_atand(x)
    assert got == pytest.approx(want, rel=4e-16, abs=1e-300)
    assert lib.gfo_atand(-x) == -got


def test_atand_is_monotonic_on_a_fine_grid():
    lib = load()
    xs = np.concatenate([np.linspace(0, 2, 4001), np.geomspace(2, 1e6, 2001)])
    ys = np.array([lib.gfo_atand(float(x)) for x in xs])
    assert np.all(np.diff(ys) >= 0)


@pytest.fixture(scope="module")
def traced():
    case = Case(configs.tiny_furnace())
    o = Oracle(case)
    o.initsv()
    o.gflow(20)
    tot = o.rad_transfer()
    f = o.download()
    yield case, tot, f
    o.close()


def test_transfer_conserves_the_emitted_energy(traced):
    case, tot, f = traced
    absorbed = (tot["qa_sum_to_open"] + tot["qa_sum_to_wall"] + tot["qa_sum_to_inlet"] + tot["qa_sum_to_exit"]
                + tot["qa_sum_to_melt"])
    assert tot["n_emitters"] > 0 and tot["qe_sum_from_open"] > 0
    assert abs(tot["qe_sum_from_open"] - absorbed) <= 1e-12 * tot["qe_sum_from_open"]
    # QA over all cells is the same energy, cell by cell
    assert f.arrays["qa"].sum() == pytest.approx(absorbed, rel=1e-12)


def test_traced_emission_equals_the_band_emission_total(traced):
    case, tot, f = traced
    assert tot["qe_sum_from_open"] == pytest.approx(tot["tot_qe_h2o_co2"], rel=1e-13)
    assert tot["tot_qe_soot"] == 0.0
    assert f.arrays["qe"].sum() == pytest.approx(tot["qe_sum_from_open"], rel=1e-13)


def test_only_hot_open_cells_emit_and_absorption_stays_in_the_box(traced):
    case, tot, f = traced
    ib = case.ibcell()[1::2, 1::2, 1::2]   # cell centres (even positions)
    qe, qa = f.arrays["qe"], f.arrays["qa"]
    assert np.all(qe[ib >= 1] == 0)
    assert np.all(qa >= 0) and np.all(qe >= 0)
    assert tot["n_emitters"] == int(np.count_nonzero(qe > 0))


@pytest.mark.parametrize("nb", [1, 2, 10])
def test_transfer_conserves_energy_for_other_band_counts(nb):
    kappa = tuple(float(k) for k in np.geomspace(0.05, 5.0, nb)) if nb > 1 else (0.7,)
    wl = tuple(float(w) for w in np.geomspace(1.5, 40.0, nb - 1)) + (1000.0,) if nb > 1 else (1000.0,)
    case = Case(configs.tiny_furnace(kappa=kappa, wl_um=wl))
    o = Oracle(case)
    o.initsv()
    o.gflow(10)
    t = o.rad_transfer()
    absorbed = sum(t[k] for k in ("qa_sum_to_open", "qa_sum_to_wall", "qa_sum_to_inlet", "qa_sum_to_exit",
                                  "qa_sum_to_melt"))
    assert t["qe_sum_from_open"] > 0
    assert abs(t["qe_sum_from_open"] - absorbed) <= 1e-12 * t["qe_sum_from_open"]
    o.close()
