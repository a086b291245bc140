"""The gas and soot band model (RAD_GAS, SOOTA in RAD0) and the minor species
restart rs####c.d, on the reference's own converged runs of TC21 case 0041
and the end-fired case 1207.

The reference wrote, at the end of each run, the gas restart rg####c.d, then
ran MSFLOW and wrote the minor species restart rs####c.d, then RAD_EMIS, whose
volume-radiation record is the last line of rad_detail####c.plt
(A0main.f90:205-233, Qrn.f90:181-197).  So the oracle's RAD0 + QRNF on the
state of those two files must print that line: the band-emission totals of
H2O/CO2 and of soot (Rad0.f90:137-148) test RAD_GAS and SOOTA, and the
emission and absorption totals (Qrn.f90:73-87) the transfer through the
band model's absorption coefficients.  The record holds 14 digits; the
oracle matches them to about 1e-14."""
import json
import lzma
import pathlib
import shutil

import numpy as np
import pytest

from gfm_gb300 import Case, abi
from gfm_gb300.solver import GfmError
from oracle.pyoracle import Oracle

GOLD = pathlib.Path(__file__).resolve().parent / "golden"
RECORD = (("tot_qe_h2o_co2", "qe_h2o_co2"), ("tot_qe_soot", "qe_soot"), ("qe_sum_from_open", "qe_from_media"),
          ("qa_sum_to_melt", "qa_melt"), ("qa_sum_to_wall", "qa_wall"), ("qa_sum_to_open", "qa_media"),
          ("qa_sum_to_exit", "qa_exit"), ("qa_sum_to_inlet", "qa_inlet"))


def converged_dir(num: str, tmp: pathlib.Path) -> pathlib.Path:
    """A case directory with the case's inputs and its end-of-run restarts."""
    gold = GOLD / f"case{num}"
    d = tmp / f"case{num}"
    d.mkdir(exist_ok=True)
    for f in gold.iterdir():
        if f.is_file() and not f.name.endswith(".xz") and not f.name.endswith(".json"):
            shutil.copyfile(f, d / f.name)
    for kind in ("rg", "rs"):
        (d / f"{kind}{num}c.d").write_bytes(lzma.decompress((gold / f"{kind}{num}c.d.xz").read_bytes()))
    return d


def reference(num: str) -> dict:
    return json.loads((GOLD / f"case{num}" / f"case{num}_reference.json").read_text())


def converged(num: str, tmp: pathlib.Path, **kw):
    d = converged_dir(num, tmp)
    case = Case.from_files(d, num, restart=True, gas_model=True, **kw)
    return case, case.read_minor(d / f"rs{num}c.d")


@pytest.mark.parametrize("num", ["0041", "1207"])
def test_band_model_reproduces_the_reference_radiation_record(tmp_path, num):
    case, minor = converged(num, tmp_path)
    ref = reference(num)["rad_detail_last"]
    assert case.summary["itr_gas"] == ref["itr_gas"]
    o = Oracle(case)
    o.minor_set(minor)
    t = o.rad_transfer()
    for mine, theirs in RECORD:
        assert t[mine] == pytest.approx(ref[theirs], rel=1e-12), (mine, t[mine], ref[theirs])
    # soot carries most of the emission in these furnaces
    assert t["tot_qe_soot"] > 5 * t["tot_qe_h2o_co2"] > 0


def test_soot_carry_over_is_exercised(tmp_path):
    """Open cells whose soot volume fraction is below 1e-14 after a cell that
    set AKLS, in RAD0's loop order: the case where SOOTA leaves AKLS as the
    previous cell set it (Rad_soot.f90:29)."""
    case, minor = converged("0041", tmp_path)
    f = case.initial_fields()
    ib = case.ibcell()
    s = (slice(1, None, 2),) * 3
    t_k = f.arrays["t"][s] * case.params.t0
    fvs = minor.smf[s] * f.arrays["dnst"][s] * case.params.dnst0 / 1.8e3
    open_ = (ib[s] <= 0) & (t_k >= 300.0)
    # loop order: I outer, K inner -> arrays are (K, J, I); transpose to (I, J, K)
    o = np.transpose(open_, (2, 1, 0)).ravel()
    v = np.transpose(fvs, (2, 1, 0)).ravel()
    setter = o & (v >= 1e-14)
    first = np.argmax(setter)
    carried = o & (v < 1e-14) & (np.arange(o.size) > first)
    assert setter.sum() > 100 and carried.sum() > 10


def test_minor_restart_round_trip(tmp_path):
    d = converged_dir("0041", tmp_path)
    case = Case.from_files(d, "0041", restart=True)
    m = case.read_minor(d / "rs0041c.d")
    assert m.itr_ms == 38700
    s = (slice(1, None, 2),) * 3
    g = m.gfm[(slice(None),) + s]
    assert g.max() <= 1.0 and g.min() >= 0.0 and m.smf.max() <= 4.0e-3
    case.write_minor(tmp_path / "again.d", m)
    assert (tmp_path / "again.d").read_bytes() == (d / "rs0041c.d").read_bytes()


def test_minor_species_inputs(tmp_path):
    case, _ = converged("0041", tmp_path)
    p = case.params
    # &INPUT of sbc0041c.dat
    assert p.gas_model == 1 and p.irstypm == 1 and p.maxms == 300 and p.bmcon == 1e-12
    assert p.aform == 0.00353 and p.aoxid == 30.0
    assert p.esf_r == 3325720 / 8.3143e3 and p.eso_r == 3325720 / 8.3143e3
    # relaxfactorc.txt and the reference's defaults
    assert (p.rfm, p.rfm_soot, p.rf_soot_form, p.rf_soot_oxid) == (0.5, 0.2, 0.3, 0.3)
    assert (p.soot_cap, p.t0_sf, p.t0_so, p.ntimesm, p.ssigma) == (4.0e-3, 0.0, 0.0, 4, 0.7)


def test_band_model_needs_the_minor_species(tmp_path):
    case, _ = converged("0041", tmp_path)
    o = Oracle(case)
    with pytest.raises(RuntimeError):
        o.rad_transfer()
    # a case without MS=1 cannot ask for the band model
    d = tmp_path / "nomin"
    d.mkdir()
    for f in converged_dir("0041", tmp_path).iterdir():
        shutil.copyfile(f, d / f.name)
    sbc = d / "sbc0041c.dat"
    sbc.write_bytes(sbc.read_bytes().replace(b"MS=1,", b"MS=0,"))
    with pytest.raises(GfmError):
        Case.from_files(d, "0041", gas_model=True)
    assert Case.from_files(d, "0041").params.gas_model == 0
