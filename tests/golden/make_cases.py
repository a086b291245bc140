"""Fixtures of the reference's shipped combustion-space cases.

  case0041  TC21 40 tpd glass furnace, burners on the left side (40x48x36
            doubled grid, 4,407 open cells), with its converged restart file
  case0040  the same furnace with another port and flue layout (4,377 cells)
  case1207  a longer end-fired furnace (154x28x30 doubled grid, 8,263 cells,
            42 inlet blocks)
  and the other shipped cases: 0020 and 0021 (the fresh starts kept in
  case0020oldrun, case0021oldrun), 0054 and 0055 (case0054-start,
  case0055-start), 0056, and 1206 (the end-fired furnace's other case)

For each case the input files are copied unchanged (gd, sbc, it and the
shared relaxfactorc.txt), and <case>_reference.json records what the
reference's own run of the case printed:

  - summary####c.txt head   open cells, melt-surface area, inlet mass flows
                            and the fuel heat input (Utility.f90:99-105), and
                            the energy in with the inlet flow, q_h_in
                            (Sbc.f90:172, printed at Utility.f90:131)
  - convg####c.plt          mean and maximum mass residual of the first 40
                            iterations of the run's fresh start
  - Tave####c.plt           mean gas and exit temperatures of its first 3
                            iterations (T_ave_calc, Utility.f90:1485-1509) and
                            the mean gas temperature of the last iteration

  - rad_detail####c.plt      the last volume-radiation record of the run
                            (Qrn.f90:181-197): its RAD0 band-emission totals
                            and the QRNF emission and absorption totals

The first 48 lines of each per-iteration log (convg, gresid, gresid_xtra,
Tave, Info and, where the run wrote them, the pre-solve gresidp and
gresid_xtrap) and the first 80 lines of summary####c.txt are copied unchanged
into logs/, as the byte-level reference of their format, and for the cases
whose restarts are kept the melt hand-over file it####m.dat written by the
run's last radiation call.  For case0041 the
converged restart file rg0041c.d and the minor species restart rs0041c.d
(written after the run's last MSFLOW, read by the RAD_EMIS of that last
rad_detail record) are stored xz-compressed.

Run from the repository root with the reference package root as argument:

    python tests/golden/make_cases.py /path/to/GFM_Source_Package_2015-08
"""
import hashlib
import json
import lzma
import pathlib
import re
import shutil
import sys

HERE = pathlib.Path(__file__).resolve().parent
# runum: (case directory in the package, keep the restart file); for 0020,
# 0021, 0054 and 0055 the directory holding the run's fresh start
CASES = {"0041": ("case0041", True), "0040": ("case0040", False), "1207": ("case1207", True),
         "0020": ("case0020oldrun", False), "0021": ("case0021oldrun", False), "0054": ("case0054-start", False),
         "0055": ("case0055-start", False), "0056": ("case0056", False), "1206": ("case1206", False)}


def data_rows(path: pathlib.Path) -> list:
    return [l.split() for l in path.read_text().splitlines() if l.strip() and not l.lstrip().startswith("#")]


def summary_value(text: str, label: str) -> float:
    m = re.search(re.escape(label) + r"\s+([-+0-9.E]+)", text)
    assert m, label
    return float(m.group(1))


def main(pkg_root: str) -> None:
    src = pathlib.Path(pkg_root) / "combustion"
    for num, (dirname, keep_rg) in CASES.items():
        case = src / dirname
        out = HERE / f"case{num}"
        out.mkdir(exist_ok=True)
        for name in (f"gd{num}c.dat", f"sbc{num}c.dat", f"it{num}t.dat"):
            shutil.copyfile(case / name, out / name)
        shutil.copyfile(src / "relaxfactorc.txt", out / "relaxfactorc.txt")
        (out / "logs").mkdir(exist_ok=True)
        for log in ("convg", "gresid", "gresidp", "gresid_xtra", "gresid_xtrap", "Tave", "Info"):
            f = case / f"{log}{num}c.plt"
            if f.exists():
                head = f.read_bytes().split(b"\r\n")[:48]
                (out / "logs" / f.name).write_bytes(b"\r\n".join(head) + b"\r\n")
        head = (case / f"summary{num}c.txt").read_bytes().split(b"\r\n")[:80]
        (out / "logs" / f"summary{num}c.txt").write_bytes(b"\r\n".join(head) + b"\r\n")
        summ = (case / f"summary{num}c.txt").read_text()
        ref = {
            "source": f"combustion/{dirname} of the reference package",
            "ncells": int(summary_value(summ, "Number of cells in combustion grid:")),
            "area_melt_surf": summary_value(summ, "Melt surface area:"),
            "fr_f": summary_value(summ, "Fuel in flow rate:"),
            "fr_ox": summary_value(summ, "Oxygen in flow rate:"),
            "fr_n2": summary_value(summ, "Nitrogen in flow rate:"),
            "fr_total": summary_value(summ, "Total in flow rate:"),
            "heat_in_fuel": summary_value(summ, "Heat value in with fuel:"),
            "q_h_in": summary_value(summ, "Energy in with flow:"),
        }
        conv = data_rows(case / f"convg{num}c.plt")
        assert int(conv[0][0]) == 1
        ref["res_mass"] = [float(r[1]) for r in conv[:40]]
        ref["res_mass_max"] = [float(r[2]) for r in conv[:40]]
        tave = data_rows(case / f"Tave{num}c.plt")
        ref["tave"] = [float(r[1]) for r in tave[:3]]
        ref["tmean_ex"] = [float(r[2]) for r in tave[:3]]
        ref["tave_iteration_last"] = int(tave[-1][0])
        ref["tave_last"] = float(tave[-1][1])
        rad = data_rows(case / f"rad_detail{num}c.plt")
        keys = ("qe_h2o_co2", "qe_soot", "qe_sum", "qe_from_media", "qa_melt", "qa_wall", "qa_media", "qa_exit",
                "qa_inlet", "qa_sum", "q_diff")
        ref["rad_detail_last"] = {"itr_gas": int(rad[-1][0]), **{k: float(v) for k, v in zip(keys, rad[-1][1:])}}
        if keep_rg:
            shutil.copyfile(case / f"it{num}m.dat", out / "logs" / f"it{num}m.dat")
            for kind in ("rg", "rs"):
                raw = (case / f"{kind}{num}c.d").read_bytes()
                (out / f"{kind}{num}c.d.xz").write_bytes(lzma.compress(raw, preset=9))
                ref[f"{kind}_sha256"] = hashlib.sha256(raw).hexdigest()
                ref[f"{kind}_bytes"] = len(raw)
        (out / f"case{num}_reference.json").write_text(json.dumps(ref, indent=1) + "\n")
        print(f"wrote {out}")


if __name__ == "__main__":
    main(sys.argv[1])
