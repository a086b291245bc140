"""Fixtures of the reference's TC21 case 0041 (40 tpd glass furnace,
combustion space with burners on the left side).

Copies the case's input files unchanged, the converged restart file
rg0041c.d xz-compressed, and writes case0041_reference.json with the numbers
the reference's own run of this case printed:

  - summary0041c.txt:3-12   open cells, melt-surface area, inlet mass flows
                            and the fuel heat input (Utility.f90:99-105)
  - summary0041c.txt:20     energy in with the inlet flow: q_h_in, the sum of
                            mdot*h over the inlet cells (Sbc.f90:172,
                            printed at Utility.f90:131)
  - Tave0041c.plt (last)    mass-weighted mean gas temperature of the last
                            iteration, 7540 (T_ave_calc, Utility.f90:1485-1509)
  - convg0041c.plt (last)   mean and maximum mass residual of that iteration

Run from the repository root with the reference package root as argument:

    python tests/golden/make_case0041.py /path/to/GFM_Source_Package_2015-08
"""
import hashlib
import json
import lzma
import pathlib
import re
import shutil
import sys

OUT = pathlib.Path(__file__).resolve().parent / "case0041"


def last_data_row(path: pathlib.Path) -> list:
    rows = [l.split() for l in path.read_text().splitlines() if l.strip() and not l.lstrip().startswith("#")]
    return rows[-1]


def summary_value(text: str, label: str) -> float:
    m = re.search(re.escape(label) + r"\s+([-+0-9.E]+)", text)
    assert m, label
    return float(m.group(1))


def main(pkg_root: str) -> None:
    src = pathlib.Path(pkg_root) / "combustion"
    case = src / "case0041"
    OUT.mkdir(exist_ok=True)
    for name in ("gd0041c.dat", "sbc0041c.dat", "it0041t.dat"):
        shutil.copyfile(case / name, OUT / name)
    shutil.copyfile(src / "relaxfactorc.txt", OUT / "relaxfactorc.txt")
    raw = (case / "rg0041c.d").read_bytes()
    (OUT / "rg0041c.d.xz").write_bytes(lzma.compress(raw, preset=9))

    summ = (case / "summary0041c.txt").read_text()
    ref = {
        "source": "combustion/case0041 of the reference package",
        "ncells": int(summary_value(summ, "Number of cells in combustion grid:")),
        "area_melt_surf": summary_value(summ, "Melt surface area:"),
        "fr_f": summary_value(summ, "Fuel in flow rate:"),
        "fr_ox": summary_value(summ, "Oxygen in flow rate:"),
        "fr_n2": summary_value(summ, "Nitrogen in flow rate:"),
        "fr_total": summary_value(summ, "Total in flow rate:"),
        "heat_in_fuel": summary_value(summ, "Heat value in with fuel:"),
        "q_h_in": summary_value(summ, "Energy in with flow:"),
        "rg_sha256": hashlib.sha256(raw).hexdigest(),
        "rg_bytes": len(raw),
    }
    tave = last_data_row(case / "Tave0041c.plt")
    ref["tave_iteration"] = int(tave[0])
    ref["tave_last"] = float(tave[1])
    conv = last_data_row(case / "convg0041c.plt")
    ref["convg_iteration"] = int(conv[0])
    ref["res_mass_last"] = float(conv[1])
    ref["res_mass_max_last"] = float(conv[2])
    (OUT / "case0041_reference.json").write_text(json.dumps(ref, indent=1) + "\n")
    print(f"wrote {OUT}")


if __name__ == "__main__":
    main(sys.argv[1])
