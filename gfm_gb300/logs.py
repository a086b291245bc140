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
