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
            if f.name.startswith(("Info", "summary")) or f.name.endswith("m.dat"):
                continue   # the run files, tested below; the melt hand-over, in test_melt_handover
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


# ---- summary and Info files (Utility.f90:47-220, A0main.f90:300-399) ---------

import re

_NUM = re.compile(r"-?\d\.\d+E[-+]\d\d|-?\d\.\d+[-+]\d{3}")


def _value(lines, label):
    for l in lines:
        if label in l:
            return float(_NUM.search(l.split(label, 1)[1]).group(0).replace("E", "e") if "E" in l else 0.0)
    raise KeyError(label)


def _header_values(text_lines):
    v = lambda lab: _value(text_lines, lab)
    n = int(re.search(r"combustion grid:\s+(\d+)", "\n".join(text_lines)).group(1))
    return dict(ncells=n, area_melt_surf=v("Melt surface area:"), fr_f=v("Fuel in flow rate:"),
                fr_ox=v("Oxygen in flow rate:"), fr_n2=v("Nitrogen in flow rate:"),
                heat_in_fuel=v("Heat value in with fuel:"))


# derived lines: sums the writer forms from its inputs, compared numerically
_DERIVED = ("Total in flow rate:", "Total energy in:", "Total energy leaving furnace:", "(sum of froms):",
            "Energy out with or from the gas", "Fuel energy out:")


def _same(got, want):
    assert len(got) == len(want), (len(got), len(want))
    for g, w in zip(got, want):
        if any(d in w for d in _DERIVED):
            assert _NUM.sub("#", g) == _NUM.sub("#", w), (g, w)
            a, b = float(_NUM.search(g).group(0)), float(_NUM.search(w).group(0))
            assert a == pytest.approx(b, rel=1e-12, abs=0), (g, w)
        else:
            assert g == w, (g, w)


@pytest.mark.parametrize("num", ["0041", "0040", "1207", "1206", "0056"])
def test_summary_file_reproduced(num):
    """The summary's inflow header and its first end-of-run energy balance
    reproduced from their values (the printed sums numerically)."""
    from gfm_gb300 import logs
    text = (GOLDEN / f"case{num}" / "logs" / f"summary{num}c.txt").read_bytes().decode()
    lines = text.split("\r\n")
    runum = re.search(r"# Case (\S+) ", lines[0]).group(1)
    head = logs.run_header(runum, "summary", **_header_values(lines[:12]))
    _same(head, lines[:12])
    # the first block: from "Run End" to the line before the next blank-blank pair
    start = lines.index("# #################   Run End   #################")
    blk = lines[start + 1:]
    end = next(i for i in range(len(blk) - 1) if blk[i].startswith("#   Mean wall temperature:")) + 1
    tail = blk[end:end + 5]
    soot = None
    if tail and tail[0].startswith("#   Maximum soot"):
        soot = (_value(tail, "Maximum soot mass fraction:"), _value(tail, "Not clipped soot mass fraction:"),
                int(tail[2].split()[-1]))
        end += 3
    cycle = None
    if blk[end:end + 2] and blk[end + 1].startswith("#   Cycle count:"):
        cycle = int(blk[end + 1].split()[-1])
        end += 2
    b = blk[:end]
    vals = {k: _value(b, lab) for k, lab in (
        ("q_h_in", "Energy in with flow:"), ("q_react", "Energy in via combustion:"),
        ("q_exhaust", "Energy out with flow:"), ("q_wall_loss", "Energy out through walls:"),
        ("q_rad_inlet", "Net radiation out inlets:"), ("q_rad_outlet", "Net radiation out outlets:"),
        ("q_melt", "Energy out to melt:"), ("qm_flame", "from flame:"), ("qm_bnds", "from surfaces:"),
        ("qm_conv", "from convection:"), ("qconv_total", "Convection to walls"),
        ("qa_sum_to_melt", "Radiation from flame to melt:"), ("qa_sum_to_wall", "Radiation from flame to walls:"),
        ("qa_sum_to_inlet", "Radiation from flame to inlets:"), ("qa_sum_to_exit", "Radiation from flame to exits:"),
        ("gfin", "Mass in:"), ("gfex", "Mass out:"), ("fuel_out", "Fuel mass out:"),
        ("tave", "Mean temperature:"), ("tmean_ex", "Mean exit temperature:"), ("avg_wall_T", "Mean wall temperature:"))}
    vals["q0_h0"] = _value(b, "Fuel energy out:") / vals["fuel_out"] if vals["fuel_out"] else 0.0
    got = logs.RUN_END[:-1] + [logs.RUN_END[-1]] + logs.end_conditions(vals, cycle_count=cycle, soot=soot)
    assert lines[start - 3:start] == ["", "", ""]
    _same(got[3:], lines[start:start + 1 + end])


@pytest.mark.parametrize("num", ["0041", "1207"])
def test_info_file_reproduced(num):
    """The Info file's header, column headings and first records from their values."""
    from gfm_gb300 import logs
    lines = (GOLDEN / f"case{num}" / "logs" / f"Info{num}c.plt").read_bytes().decode().split("\r\n")
    runum = re.search(r"# Case (\S+) ", lines[0]).group(1)
    head = logs.run_header(runum, "info", **_header_values(lines[:13]))
    _same(head, lines[:13])
    assert lines[13:16] == ["", logs.INFO_COLUMNS, ""]
    for l in lines[16:40]:
        f = l.split()
        rec = logs.info_record(int(f[0]), *[float(x) for x in f[1:]])
        assert rec == l


def test_run_files_of_an_oracle_run(tmp_path):
    """RunFiles over a short run of TC21 case 0041 (the oracle, with a
    volume transfer and the wall exchange at its end): the header equals the
    reference's from the case's own start-up figures, one Info record per
    iteration, and the energy balance with the exchange's totals."""
    from oracle.pyoracle import Oracle
    case = read_case("0041", tmp_path, kappa=[0.5] * 16, wall_sink=True)
    s = case.summary
    hdr = dict(ncells=s["ncells"], area_melt_surf=s["area_melt_surf"], fr_f=s["fr_f"], fr_ox=s["fr_ox"],
               fr_n2=s["fr_n2"], heat_in_fuel=s["heat_in_fuel"])
    runs = tmp_path / "run"
    runs.mkdir()
    rf = logs.RunFiles(runs, "0041", hdr)
    o = Oracle(case)
    o.initsv()
    o.wall_setup()
    for _ in range(2):
        st = o.gflow(1)[0]
        rf.iteration(st["itr_gas"], q_h_in=s["q_h_in"], q_react=st["q_react"], q_melt=0.0,
                     q_exhaust=st["q_exhaust"], q_wall_loss=0.0, q_rad_openings=0.0, q_incident_total=0.0,
                     qconv_total=st["q_conv_total"])
    rad = o.rad_transfer()
    w = o.wall_totals()
    vals = {"q_h_in": s["q_h_in"], "q_react": st["q_react"], "q_exhaust": st["q_exhaust"], "q_melt": w["q_melt"],
            "q_wall_loss": w["q_wall_loss"], "q_rad_inlet": w["q_rad_inlet"], "q_rad_outlet": w["q_rad_outlet"],
            "qm_flame": w["qm_flame"], "qm_bnds": w["qm_bnds"], "qm_conv": w["qm_conv"],
            "qconv_total": w["qconv_total"], "qa_sum_to_melt": rad["qa_sum_to_melt"],
            "qa_sum_to_wall": rad["qa_sum_to_wall"], "qa_sum_to_inlet": rad["qa_sum_to_inlet"],
            "qa_sum_to_exit": rad["qa_sum_to_exit"], "gfin": st["gfin"], "gfex": st["gfex"], "fuel_out": 0.0,
            "q0_h0": 0.0, "tave": st["tave"], "tmean_ex": st["tmean_ex"], "avg_wall_T": w["avg_wall_T"]}
    rf.end(vals)
    o.close()
    summ = (runs / "summary0041c.txt").read_bytes().decode().split("\r\n")
    ref = (GOLDEN / "case0041" / "logs" / "summary0041c.txt").read_bytes().decode().split("\r\n")
    # the reference run's runum in the header is its own case's; the rest must agree
    _same(summ[1:12], ref[1:12])
    info = (runs / "Info0041c.plt").read_bytes().decode().split("\r\n")
    assert info[13:16] == ["", logs.INFO_COLUMNS, ""]
    assert [int(l.split()[0]) for l in info[16:18]] == [1, 2]
    assert any(l.startswith("#   Mean wall temperature:") for l in summ)
