"""The .plt logs (gfm_gb300.logs) against the reference's own: every stored
log head of the three fixture cases (tests/golden/case*/logs, the first 48
lines of the files the reference's runs wrote) is rewritten byte for byte
from its values, and a run of the oracle writes files with the same headers
and record layout."""
import pathlib

import pytest

from gfm_gb300 import logs

from .test_case_files import CASES, read_case

GOLDEN = pathlib.Path(__file__).parent / "golden"
SPEC = {"convg": (7, 25, 16), "gresid": (7, 24, 16), "gresidp": (7, 24, 16), "gresid_xtra": (7, 24, 16),
        "gresid_xtrap": (7, 24, 16), "Tave": (5, 22, 14)}


def stored_logs():
    for num in CASES:
        for f in sorted((GOLDEN / f"case{num}" / "logs").iterdir()):
            yield num, f


def split_record(line: str, iw: int, w: int) -> tuple:
    body = line[iw:]
    return int(line[:iw]), [float(body[i:i + w]) for i in range(0, len(body), w)]


@pytest.mark.parametrize("num,path", list(stored_logs()), ids=lambda x: getattr(x, "name", x))
def test_reference_log_rewritten_byte_for_byte(num, path):
    name = path.name[: -len(f"{num}c.plt")]
    iw, w, d = SPEC[name]
    lines = path.read_bytes().decode().split("\r\n")
    hdr = logs._HEADERS[name]
    assert tuple(lines[:len(hdr)]) == hdr
    rows = [l for l in lines[len(hdr):] if l.strip()]
    assert len(rows) >= 40
    for l in rows:
        it, vals = split_record(l, iw, w)
        assert logs.fortran_i(it, iw) + "".join(logs.fortran_e(v, w, d) for v in vals) == l


def test_fortran_e_edges():
    assert logs.fortran_e(0.0, 24, 16) == "  0.0000000000000000E+00"
    assert logs.fortran_e(-1.5, 24, 16) == " -0.1500000000000000E+01"
    assert logs.fortran_e(1e-16, 24, 16) == "  0.1000000000000000E-15"
    assert logs.fortran_e(1.0e-120, 24, 16) == "  0.1000000000000000-119"
    assert logs.fortran_e(9.99999999999999999e5, 22, 14) == "  0.10000000000000E+07"


def test_oracle_run_writes_the_reference_layout(tmp_path):
    from oracle.pyoracle import Oracle
    case = read_case("0041", tmp_path)
    o = Oracle(case)
    o.initsv()
    out = tmp_path / "run"
    out.mkdir()
    with logs.PlotLogs(out, "0041") as pl:
        for _ in range(3):
            pl.write(o.gflow(1)[0])
    o.close()
    for name, (iw, w, d) in SPEC.items():
        got = (out / f"{name}0041c.plt").read_bytes().decode().split("\r\n")
        hdr = logs._HEADERS[name]
        assert tuple(got[:len(hdr)]) == hdr
        rows = [l for l in got[len(hdr):] if l]
        assert [split_record(l, iw, w)[0] for l in rows] == [1, 2, 3]
        ref = GOLDEN / "case0041" / "logs" / f"{name}0041c.plt"
        if ref.exists():   # same record width as the reference's
            ref_rows = [l for l in ref.read_bytes().decode().split("\r\n")[len(hdr):] if l]
            assert len(rows[0]) == len(ref_rows[0])
    # appending on a restart keeps the header once
    with logs.PlotLogs(out, "0041", restart=True) as pl:
        pl.write(dict(o_stats := {"itr_gas": 4, "res_mass": 0.1, "res_mass_max": 1.0, "gf_resid": [1e-3] * 10,
                                  "gf_resid_pre": [1e-3] * 10, "p_resid": 1e-3, "p_resid_pre": 1e-3,
                                  "u_resid": [1e-6] * 3, "u_resid_pre": [1e-6] * 3, "tave": 1500.0,
                                  "tmean_ex": 1500.0}))
    txt = (out / "convg0041c.plt").read_bytes().decode()
    assert txt.count("PlotData") == 1 and txt.rstrip().endswith("0.1000000000000000E+01")
