"""The combustion side's hand-over to the melt domain, it####m.dat (QRN_PRN,
Qrn.f90:363-392): the writer against the reference's own files, byte for
byte, and the wall exchange's melt-surface heat flux, mean wall temperature
and heat into the melt against the file TC21 case 0041's run wrote after its
last radiation call.

The oracle starts that exchange from the cells' temperatures and without the
gas's convective wall flux of the last iteration (neither is in the restart
files); from there it reaches the reference's mean wall temperature to 4e-7
and its heat into the melt to 3e-6, and every patch's flux to 5e-4 of the
largest (the file keeps four digits)."""
import pathlib

import numpy as np
import pytest

from gfm_gb300 import logs
from oracle.pyoracle import Oracle

from .test_oracle_gas import converged

GOLD = pathlib.Path(__file__).resolve().parent / "golden"


def _coords(case):
    g = case.grid
    return np.ctypeslib.as_array(g.x, shape=(g.mp,)).copy(), np.ctypeslib.as_array(g.r, shape=(g.np,)).copy()


@pytest.mark.parametrize("num", ["0041", "1207"])
def test_melt_flux_file_round_trip(tmp_path, num):
    case, _ = converged(num, tmp_path)
    x, r = _coords(case)
    raw = (GOLD / f"case{num}" / "logs" / f"it{num}m.dat").read_bytes()
    v = logs.read_melt_flux_file(raw, case.mp, case.np)
    assert logs.melt_flux_file(x, r, v["qrs"], v["avg_wall_T"], v["tmax_c"], v["q_melt"], v["itn"]) == raw


def test_wall_exchange_reproduces_the_melt_handover(tmp_path):
    case, minor = converged("0041", tmp_path, wall_sink=True)
    ref = logs.read_melt_flux_file((GOLD / "case0041" / "logs" / "it0041m.dat").read_bytes(), case.mp, case.np)
    o = Oracle(case)
    o.initsv()
    o.minor_set(minor)
    o.wall_setup()
    o.rad_transfer()
    w = o.wall_totals()
    assert w["avg_wall_T"] == pytest.approx(ref["avg_wall_T"], rel=1e-6)
    assert w["q_melt"] == pytest.approx(ref["q_melt"], rel=1e-5)
    t = case.initial_fields().arrays["t"][1::2, 1::2, 1::2] * case.params.t0
    assert t.max() == pytest.approx(ref["tmax_c"], rel=1e-14)
    pl = o.wall_patch_list()
    qrs = o.patch_array("qrs")
    mine = {(int(p[1]), int(p[2])): q for p, q in zip(pl, qrs) if p[0] == 4}
    assert set(mine) == {k for k, v in ref["qrs"].items() if v != 0.0}
    top = max(abs(v) for v in ref["qrs"].values())
    assert max(abs(mine.get(k, 0.0) - v) for k, v in ref["qrs"].items()) < 1e-3 * top
    # the file written from this exchange reads back as the reference's, to its digits
    x, r = _coords(case)
    again = logs.read_melt_flux_file(logs.melt_flux_file(x, r, mine, w["avg_wall_T"], t.max(), w["q_melt"]),
                                     case.mp, case.np)
    assert again["avg_wall_T"] == pytest.approx(ref["avg_wall_T"], rel=1e-6)
    assert max(abs(again["qrs"][k] - v) for k, v in ref["qrs"].items()) < 1e-3 * top
