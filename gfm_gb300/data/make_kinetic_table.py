"""Copy the integral-reaction kinetics table into the package.

The reference reads `kinetic.d` (combustion/Kinetic.d, read by
allocate_large_gas_phase_arrays, combustion/Code/Setup.f90:867-888): two
tables of 100 rows (RTIM DELRT HRT, then DELR TIMED HRD) of measured reaction
progress data.  The numbers are physical data that must be identical for the
fuel source term (Source.f90:197-206) to match, so they are copied verbatim
(line endings normalised).  Run from the repository root:

    python gfm_gb300/data/make_kinetic_table.py /path/to/GFM_Source_Package_2015-08
"""
import pathlib
import sys


def main(pkg_root: str) -> None:
    src = pathlib.Path(pkg_root) / "combustion" / "Kinetic.d"
    dst = pathlib.Path(__file__).with_name("kinetic.d")
    lines = src.read_text().splitlines()
    rows = [" ".join(l.split()) for l in lines if l.strip()]
    assert len(rows) == 202, len(rows)
    dst.write_text("\n".join(rows) + "\n")
    print(f"wrote {dst} ({len(rows)} lines)")


if __name__ == "__main__":
    main(sys.argv[1])
