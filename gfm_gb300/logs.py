"""Per-iteration logs in the reference's .plt formats, the files its RunPlot
tool reads from a case directory.

Each file starts as the reference's *_file_init routine starts it, a fresh
file for a fresh start and appended to on a restart (Utility.f90:272-291,
507-666, 1072-1081).  Each iteration adds one record written with the edit
descriptors of the reference's WRITE statements:

  convg####c.plt        (i7,4e25.16)  itr_gas, res_mass, res_mass_max
                                      (Sphase.f90:53)
  gresid####c.plt       (i7,5e24.16)  itr_gas, h, p, u, v, w residuals
                                      (Gflow.f90:260)
  gresidp####c.plt      (i7,5e24.16)  the same before the solves (Gflow.f90:263)
  gresid_xtra####c.plt  (i7,6e24.16)  fuel, O2, CO2, N2, k, epsilon residuals
                                      (Gflow.f90:268); the header names the
                                      last two columns "Epsilon" and "k"
  gresid_xtrap####c.plt (i7,6e24.16)  the same before the solves (Gflow.f90:271)
  Tave####c.plt         (i5,2e22.14)  itr_gas, mean gas and exit temperature
                                      (Gflow.f90:401; the three-column form
                                      after the first full radiation call adds
                                      the mean wall temperature, which comes
                                      from the wall radiosity exchange)

List-directed header lines start with a blank, as the reference's compiler
writes them, and lines end in CR-LF as in the shipped case directories.

The run files of the GUI's energy-balance views are written here too:

  summary####c.txt   the inflow header (summary_file_init, Utility.f90:95-
                     108), then at the end of a run a "Run End" line and the
                     energy balance (A0main.f90:315-320,
                     sum_info_file_end_conditions, Utility.f90:124-220)
  Info####c.plt      the same header (Info_file_init, Utility.f90:47-67),
                     one energy record per iteration ((1x,i5,8e22.14),
                     track_energy, A0main.f90:371-399) and the energy balance
                     at the end of the run (A0main.f90:300-312)

and the combustion side's hand-over to the melt domain:

  it####m.dat        the melt-surface heat flux after a radiation call, with
                     the mean wall temperature, the largest gas temperature
                     and the heat into the melt (QRN_PRN, Qrn.f90:363-392);
                     the melt domain reads it and writes it####t.dat back
"""
from __future__ import annotations

import pathlib


def fortran_e(v: float, w: int, d: int) -> str:
    """Fortran Ew.d output of a real: a 0.ddd mantissa of d digits and a
    signed two-digit exponent (three digits without the E beyond 99),
    right-justified in w columns."""
    if v != v:
        return "NaN".rjust(w)
    if v in (float("inf"), float("-inf")):
        return ("-Infinity" if v < 0 else "Infinity").rjust(w)
    sign = "-" if v < 0 or (v == 0 and str(v).startswith("-")) else ""
    a = abs(v)
    if a == 0:
        mant, exp = "0" * d, 0
    else:
        s = f"{a:.{d - 1}e}"              # d significant digits, rounded to nearest
        digits, e = s.split("e")
        mant = digits.replace(".", "")
        exp = int(e) + 1
    if abs(exp) <= 99:
        tail = f"E{'+' if exp >= 0 else '-'}{abs(exp):02d}"
    else:
        tail = f"{'+' if exp >= 0 else '-'}{abs(exp):03d}"
    return f"{sign}0.{mant}{tail}".rjust(w)


def fortran_i(n: int, w: int) -> str:
    return str(int(n)).rjust(w)


_ITER = "# Iter "
_HEADERS = {
    "convg": (" # Combustion space mean and max mass residual - log plot", " # PlotData",
              " # iteration  average mass residual  max mass residual"),
    "gresid": (" # Mean residuals - log plot", " # PlotData ", "",
               _ITER + "        Enthalpy        " + "        Pressure        " + "       x-momentum       "
               + "       y-momentum       " + "       z-momentum       ", ""),
    "gresidp": (" # Mean residuals (pre-solve) - log plot", " # PlotData ", "",
                _ITER + "      Pre-Enthalpy      " + "      Pre-Pressure      " + "     Pre-x-momentum     "
                + "     Pre-y-momentum     " + "     Pre-z-momentum     ", ""),
    "gresid_xtra": (" # Mean residuals: major species, k-epsilon - log plot", " # PlotData ", "",
                    _ITER + "        Fuel            " + "        O2              " + "        CO2             "
                    + "        N2              " + "        Epsilon         " + "        k               ", ""),
    "gresid_xtrap": (" # Mean residuals: major species, k-epsilon (pre-solve) - log plot", " # PlotData ", "",
                     _ITER + "      Pre-Fuel          " + "      Pre-O2            " + "      Pre-CO2           "
                     + "      Pre-N2            " + "      Pre-Epsilon       " + "      Pre-k             ", ""),
    "Tave": (" # Combustion space mean temperature", " # PlotData ", "",
             "# Iter      " + "Mean Gas Temp (K)     " + "Mean Exit Temp        " + "Mean Wall Temp", ""),
}


def records(stats: dict) -> dict:
    """The record of each log for one iteration's statistics (the dict of
    gfm_iter_stats), formatted as the reference writes it."""
    it = stats["itr_gas"]
    r, rp = stats["gf_resid"], stats["gf_resid_pre"]

    def row(iw: int, w: int, d: int, vals) -> str:
        return fortran_i(it, iw) + "".join(fortran_e(v, w, d) for v in vals)

    # GF index L-1: 0 fuel, 1 O2, 2 h, 3 k, 4 eps, 5 CO2, 6 N2
    return {
        "convg": row(7, 25, 16, (stats["res_mass"], stats["res_mass_max"])),
        "gresid": row(7, 24, 16, (r[2], stats["p_resid"], *stats["u_resid"])),
        "gresidp": row(7, 24, 16, (rp[2], stats["p_resid_pre"], *stats["u_resid_pre"])),
        "gresid_xtra": row(7, 24, 16, (r[0], r[1], r[5], r[6], r[3], r[4])),
        "gresid_xtrap": row(7, 24, 16, (rp[0], rp[1], rp[5], rp[6], rp[3], rp[4])),
        "Tave": row(5, 22, 14, (stats["tave"], stats["tmean_ex"])),
    }


class PlotLogs:
    """The .plt logs of one case directory: `write(stats)` after every
    iteration, `close()` at the end of the run."""

    def __init__(self, case_dir, runum: str, restart: bool = False, newline: str = "\r\n",
                 names=("convg", "gresid", "gresidp", "gresid_xtra", "gresid_xtrap", "Tave")):
        self.nl = newline
        self.fh = {}
        for n in names:
            path = pathlib.Path(case_dir) / f"{n}{runum}c.plt"
            if restart and path.exists():
                self.fh[n] = open(path, "a", newline="")
            else:
                self.fh[n] = open(path, "w", newline="")
                self.fh[n].write(self.nl.join(_HEADERS[n]) + self.nl)

    def write(self, stats: dict) -> None:
        rec = records(stats)
        for n, f in self.fh.items():
            f.write(rec[n] + self.nl)

    def close(self) -> None:
        for f in self.fh.values():
            f.close()
        self.fh = {}

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


# ---- summary and Info files ---------------------------------------------------

def tabbed(*fields) -> str:
    """One record of T-positioned fields: (column, text) pairs, the column
    1-based as in a Tn edit descriptor, text placed from that column."""
    line: list = []
    for col, text in fields:
        pos = col - 1
        if len(line) < pos:
            line.extend(" " * (pos - len(line)))
        line[pos:pos + len(text)] = list(text)
    return "".join(line)


def run_header(runum: str, kind: str, ncells: int, area_melt_surf: float, fr_f: float, fr_ox: float,
               fr_n2: float, heat_in_fuel: float) -> list:
    """The lines summary_file_init ("Summary Data") or Info_file_init
    ("Information") writes on a fresh start (Utility.f90:61-67, 99-108)."""
    title = {"summary": "Summary Data", "info": "Information"}[kind]
    e = lambda v: fortran_e(v, 25, 14)
    lines = [f"# Case {runum} {title} for Simulation and Evolving Global Energy Distribution", "",
             tabbed((1, "# "), (5, "Number of cells in combustion grid:"), (40, fortran_i(ncells, 7))),
             tabbed((1, "# "), (5, "Melt surface area: "), (38, e(area_melt_surf) + " m^2")), "",
             tabbed((1, "# "), (5, "Fuel in flow rate: "), (38, e(fr_f) + " kg/s")),
             tabbed((1, "# "), (5, "Oxygen in flow rate: "), (38, e(fr_ox) + " kg/s")),
             tabbed((1, "# "), (5, "Nitrogen in flow rate: "), (38, e(fr_n2) + " kg/s")),
             tabbed((1, "# "), (5, "Total in flow rate: "), (38, e(fr_n2 + fr_ox + fr_f) + " kg/s")), "",
             tabbed((1, "# "), (5, "Heat value in with fuel: "), (38, e(heat_in_fuel) + " W")),
             "  "]
    if kind == "info":
        lines.append("# PlotData")
    return lines


INFO_COLUMNS = ("# iter      " + "h flow in             " + "q reaction            " + "q melt                "
                + "q exhaust             " + "q wall loss         " + "q rad opening loss      "
                + "q from media          " + "q gas to wall")


def info_record(itr_gas: int, q_h_in: float, q_react: float, q_melt: float, q_exhaust: float,
                q_wall_loss: float, q_rad_openings: float, q_incident_total: float, qconv_total: float) -> str:
    """One iteration's record of the Info file (track_energy, A0main.f90:392-399)."""
    vals = (q_h_in, q_react, q_melt, q_exhaust, q_wall_loss, q_rad_openings, q_incident_total, qconv_total)
    return " " + fortran_i(itr_gas, 5) + "".join(fortran_e(v, 22, 14) for v in vals)


def end_conditions(v: dict, cycle_count=None, soot=None) -> list:
    """sum_info_file_end_conditions (Utility.f90:124-220) from the run's end
    values: q_react, q_h_in, q_exhaust, q_melt, q_wall_loss, q_rad_inlet,
    q_rad_outlet, qm_flame, qm_bnds, qm_conv, qconv_total, qa_sum_to_melt,
    qa_sum_to_wall, qa_sum_to_inlet, qa_sum_to_exit, gfin, gfex, fuel_out,
    q0_h0 (Q0*H_0, the fuel heat per unit fuel mass), tave, tmean_ex,
    avg_wall_T.  `soot` = (smf_max, smf_max_noclip, clipped count) and
    `cycle_count` add the lines the reference writes when they apply."""
    e = lambda x: fortran_e(x, 25, 14)

    def row(ind, label, col, x, unit):
        return tabbed((1, "# "), (ind, label), (col, e(x) + unit))

    q_in = v["q_react"] + v["q_h_in"]
    out = v["q_exhaust"] + v["q_melt"] + v["q_wall_loss"] + v["q_rad_inlet"] + v["q_rad_outlet"]
    gas_out = (v["q_exhaust"] + v["qconv_total"] + v["qm_conv"] + v["qa_sum_to_melt"] + v["qa_sum_to_wall"]
               + v["qa_sum_to_inlet"] + v["qa_sum_to_exit"])
    L = ["", "# Energy Balance on Exterior Walls", "# --------------------------------", "",
         row(5, "Total energy in:", 36, q_in, " W"),
         row(9, "Energy in with flow:", 40, v["q_h_in"], " W"),
         row(9, "Energy in via combustion:", 40, v["q_react"], " W"), "",
         row(5, "Total energy leaving furnace:", 36, out, " W"),
         row(9, "Energy out with flow:", 40, v["q_exhaust"], " W"),
         row(9, "Energy out through walls:", 40, v["q_wall_loss"], " W"),
         row(9, "Net radiation out inlets:", 40, v["q_rad_inlet"], " W"),
         row(9, "Net radiation out outlets:", 40, v["q_rad_outlet"], " W"),
         row(9, "Energy out to melt:", 40, v["q_melt"], " W"),
         row(13, "from flame:", 44, v["qm_flame"], " W"),
         row(13, "from surfaces:", 44, v["qm_bnds"], " W"),
         row(13, "from convection:", 44, v["qm_conv"], " W"),
         row(13, "(sum of froms):", 44, v["qm_flame"] + v["qm_bnds"] + v["qm_conv"], " W"),
         "", "# Gas Energy Balance", "# --------------------------------", "",
         row(5, "Total energy in:", 36, q_in, " W"),
         row(9, "Energy in with flow:", 40, v["q_h_in"], " W"),
         row(9, "Energy in via combustion:", 40, v["q_react"], " W"), "",
         row(5, "Energy out with or from the gas:", 36, gas_out, " W"),
         row(9, "Energy out with flow", 40, v["q_exhaust"], " W"),
         row(9, "Convection to walls", 40, v["qconv_total"], " W"),
         row(9, "Convection to melt surface", 40, v["qm_conv"], " W"),
         row(9, "Radiation from flame to melt:", 40, v["qa_sum_to_melt"], " W"),
         row(9, "Radiation from flame to walls:", 40, v["qa_sum_to_wall"], " W"),
         row(9, "Radiation from flame to inlets:", 40, v["qa_sum_to_inlet"], " W"),
         row(9, "Radiation from flame to exits:", 40, v["qa_sum_to_exit"], " W"),
         "", "# --------------------------------",
         "", row(5, "Mass in:", 36, v["gfin"], " kg/s"),
         row(5, "Mass out:", 36, v["gfex"], " kg/s"),
         "", row(5, "Fuel mass out:", 36, v["fuel_out"], " kg/s"),
         row(5, "Fuel energy out:", 36, v["fuel_out"] * v["q0_h0"], " W"),
         "", row(5, "Mean temperature:", 36, v["tave"], " K"),
         row(5, "Mean exit temperature:", 36, v["tmean_ex"], " K"),
         row(5, "Mean wall temperature:", 36, v["avg_wall_T"], " K")]
    if soot is not None:
        L += [tabbed((1, "# "), (5, "Maximum soot mass fraction:"), (36, e(soot[0]))),
              tabbed((1, "# "), (5, "Not clipped soot mass fraction:"), (36, e(soot[1]))),
              tabbed((1, "# "), (5, "Number of cells clipped:"), (36, fortran_i(soot[2], 9)))]
    if cycle_count is not None:
        L += ["", tabbed((1, "# "), (5, "Cycle count:"), (36, fortran_i(cycle_count, 5)))]
    return L


RUN_END = ["", "", "", "# #################   Run End   #################", ""]


class RunFiles:
    """summary####c.txt and Info####c.plt of one run in a case directory:
    the inflow header at the start (appended to on a restart, as the
    reference does when the file exists and IRSTYP > 0), `iteration(...)`
    after every iteration, `end(values)` at the end of the run."""

    def __init__(self, case_dir, runum: str, header: dict, restart: bool = False, newline: str = "\r\n"):
        self.nl = newline
        self.fh = {}
        self.info_started = False
        for kind, name in (("summary", f"summary{runum}c.txt"), ("info", f"Info{runum}c.plt")):
            path = pathlib.Path(case_dir) / name
            if restart and path.exists():
                self.fh[kind] = open(path, "a", newline="")
            else:
                self.fh[kind] = open(path, "w", newline="")
                self._lines(kind, run_header(runum, kind, **header))

    def _lines(self, kind: str, lines) -> None:
        self.fh[kind].write("".join(l + self.nl for l in lines))

    def iteration(self, itr_gas: int, **q) -> None:
        """One Info record (track_energy); the column headings before the first."""
        if not self.info_started:
            self._lines("info", ["", INFO_COLUMNS, ""])
            self.info_started = True
        self._lines("info", [info_record(itr_gas, **q)])

    def end(self, values: dict) -> None:
        self._lines("info", [INFO_COLUMNS] + end_conditions(values))
        self._lines("summary", RUN_END + end_conditions(values))
        self.close()

    def close(self) -> None:
        for f in self.fh.values():
            f.close()
        self.fh = {}



# ---- it####m.dat: the heat flux into the melt ------------------------------------
_MELT_LABELS = ("              Distribution indicator", "  Mean Wall Temperature in Combustion Space (K)",
                "  Max Temperature in Combustion Space (K)", "  Heat Transfer to Melter (W)")


def list_real(v: float) -> str:
    """The reference compiler's list-directed output of a REAL(8) of
    magnitude 0.1 to 1e15: fifteen significant digits in a 19-column F field
    and six trailing blanks."""
    import math
    a = abs(v)
    if not (0.1 <= a < 1.0e15):
        return f"{v:25.15E}"
    e = int(math.floor(math.log10(a)))
    for ee in (e, e + 1):
        t = f"{a:.{max(0, 14 - ee)}f}"
        if len(t.replace(".", "").lstrip("0")) <= 15 or ee == e + 1:
            break
    return (("-" if v < 0 else "") + t).rjust(19) + " " * 6


def melt_flux_file(x, r, qrs, avg_wall_T: float, tmax_c: float, q_melt: float, itn: int = 1) -> bytes:
    """it####m.dat as QRN_PRN writes it (Qrn.f90:363-392).  x and r are the
    doubled grid's X(1..MP) and R(1..NP) (0-based arrays), qrs[(I, J)] the
    melt-surface heat flux (W/m2) at the even positions that have one (0
    elsewhere).  Returns the bytes, CR-LF line ends."""
    mp, np_ = len(x), len(r)
    lines = [fortran_i(itn, 12) + " " + _MELT_LABELS[0]]
    for v, lab in zip((avg_wall_T, tmax_c, q_melt), _MELT_LABELS[1:]):
        lines.append(list_real(v) + lab)
    lines += ["", " " * 9 + "Surface Radiation Heat Flux (W/m**2)"]
    j1 = 2
    while True:
        j2 = min(j1 + 20, np_)
        js = range(j1, j2 + 1, 2)
        lines += ["", "    X  /  Y" + "".join(f"{r[j - 1]:11.3f}" for j in js)]
        for i in range(2, mp + 1, 2):
            lines.append(f"{x[i - 1]:11.3f}" + "".join(fortran_e(float(qrs.get((i, j), 0.0)), 11, 4) for j in js))
        j1 = j2 + 2
        if j1 > np_:
            break
    return ("\r\n".join(lines) + "\r\n").encode()


def read_melt_flux_file(data: bytes, mp: int, np_: int) -> dict:
    """The numbers of an it####m.dat: itn, avg_wall_T, tmax_c, q_melt and
    qrs[(I, J)] in the file's column order."""
    rows = data.decode().split("\r\n")
    out = {"itn": int(rows[0].split()[0]), "avg_wall_T": float(rows[1].split()[0]),
           "tmax_c": float(rows[2].split()[0]), "q_melt": float(rows[3].split()[0]), "qrs": {}}
    k, j1 = 6, 2
    while j1 <= np_:
        j2 = min(j1 + 20, np_)
        js = list(range(j1, j2 + 1, 2))
        k += 2   # the blank line and the X / Y header
        for i in range(2, mp + 1, 2):
            vals = [float(rows[k][11 + 11 * n: 22 + 11 * n]) for n in range(len(js))]
            for j, v in zip(js, vals):
                out["qrs"][(i, j)] = v
            k += 1
        j1 = j2 + 2
    return out
