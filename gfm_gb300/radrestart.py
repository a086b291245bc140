"""The radiation restart rr####c.d: what RAD_EMIS writes after each full
radiation call (Rad_emis.f90:289-350) and rad_emis_rr reads back on a
restart (Rad_emis.f90:17-110).

The file is Fortran sequential unformatted (4-byte little-endian record
lengths around each record), in this order:

  QE, QA, QL (MZ,NZ,LZ) and wall_rad_T (MP,NP,LP), I fastest;
  QEG0, QEG_G, QEG_W, QEG_S, QEG_IO, QES0 (the reader takes the first five);
  QEW0, QEW_G, QEW_W, QEW_S, QEW_IO;  QES0, SVF_R, QA_S0, QA_S1, QLS_G, QLS_A;
  q_melt, q_wall_loss;  q_exhaust, q_rad_inlet, q_rad_outlet;
  b_cnt, preset_vf, iterw, iwall_count, imelt_count, inlet_count, iexit_count
  (one 4-byte integer a record);
  wall, melt, inlet, exit and boundary area totals, the five incident
  totals, qconv_total (one double a record);  aoxid, aform;  avg_wall_T;
  b_typ, b_i, b_j, b_k, b_orient, b_direct (2-byte integers, b_cnt each);
  patch_area, b_face_area;  with preset_vf = 1 vf (b_cnt x b_cnt, vf(n,m)
  with n fastest) and vf_sum;  radiosity, emis, q_amb, q_conv, qc, qeb, b_T;
  bc_i, bc_j, bc_k, b_exh (2-byte integers).

`collect` forms that content from a handle after a volume transfer with the
wall exchange, `write` and `read` move it to and from the file, and
`restore` gives a new handle the wall state a restart continues from.  The
fields part (QE, QA and wall_rad_T into T and H) is read with the case
(`Case.from_files(..., restart=True, rad_restart=...)`).
"""
from __future__ import annotations

import math
import pathlib
import struct

import numpy as np

TOTALS_G = ("qeg0", "qeg_g", "qeg_w", "qeg_s", "qeg_io")
TOTALS_W = ("qew0", "qew_g", "qew_w", "qew_s", "qew_io")
TOTALS_S = ("qes0", "svf_r", "qa_s0", "qa_s1", "qls_g", "qls_a")
COUNTS = ("b_cnt", "preset_vf", "iterw", "iwall_count", "imelt_count", "inlet_count", "iexit_count")
SCALARS = ("wall_area_total", "melt_area_total", "inlet_area_total", "exit_area_total", "boundary_area_total",
           "q_incident_total", "q_incident_wall", "q_incident_inlet", "q_incident_exit", "q_incident_melt",
           "qconv_total")
PATCH_INT = ("b_typ", "b_i", "b_j", "b_k", "b_orient", "b_direct")
PATCH_REAL = ("radiosity", "emis", "q_amb", "q_conv", "qc", "qeb", "b_T")
CENTRE_INT = ("bc_i", "bc_j", "bc_k", "b_exh")


class RadRestartError(ValueError):
    """A file that does not hold the records of a radiation restart (the
    reference stops there: "unable to read radiation restart file")."""


def _records(raw: bytes) -> list[bytes]:
    out, p = [], 0
    while p < len(raw):
        if p + 4 > len(raw):
            raise RadRestartError("truncated record marker")
        (n,) = struct.unpack_from("<I", raw, p)
        if p + 8 + n > len(raw) or struct.unpack_from("<I", raw, p + 4 + n)[0] != n:
            raise RadRestartError(f"bad record at byte {p}")
        out.append(raw[p + 4:p + 4 + n])
        p += 8 + n
    return out


def _rec(payload: bytes) -> bytes:
    n = struct.pack("<I", len(payload))
    return n + payload + n


def write(path, d: dict) -> None:
    """Writes `d` (the keys `collect` forms) in RAD_EMIS's record order."""
    f8 = lambda *v: np.asarray(v, dtype="<f8").tobytes()
    parts = [np.ascontiguousarray(d[k], dtype="<f8").tobytes() for k in ("qe", "qa", "ql", "wall_rad_T")]
    parts.append(f8(*(d[k] for k in TOTALS_G), d["qes0"]))
    parts.append(f8(*(d[k] for k in TOTALS_W)))
    parts.append(f8(*(d[k] for k in TOTALS_S)))
    parts.append(f8(d["q_melt"], d["q_wall_loss"]))
    parts.append(f8(d["q_exhaust"], d["q_rad_inlet"], d["q_rad_outlet"]))
    parts += [struct.pack("<i", int(d[k])) for k in COUNTS]
    parts += [f8(d[k]) for k in SCALARS]
    parts.append(f8(d["aoxid"], d["aform"]))
    parts.append(f8(d["avg_wall_T"]))
    parts += [np.asarray(d[k], dtype="<i2").tobytes() for k in PATCH_INT]
    parts += [np.asarray(d[k], dtype="<f8").tobytes() for k in ("patch_area", "b_face_area")]
    if int(d["preset_vf"]) == 1:
        parts.append(np.asarray(d["vf"], dtype="<f8").tobytes(order="F"))   # vf(n,m), n fastest
        parts.append(np.asarray(d["vf_sum"], dtype="<f8").tobytes())
    parts += [np.asarray(d[k], dtype="<f8").tobytes() for k in PATCH_REAL]
    parts += [np.asarray(d[k], dtype="<i2").tobytes() for k in CENTRE_INT]
    pathlib.Path(path).write_bytes(b"".join(_rec(p) for p in parts))


def read(src, mp: int, np_: int, lp: int) -> dict:
    """The records of an rr file (a path or its bytes) in rad_emis_rr's
    order; QE, QA and QL come back as (LZ, NZ, MZ) arrays, wall_rad_T as
    (LP, NP, MP), vf as vf[n, m]."""
    raw = src if isinstance(src, (bytes, bytearray)) else pathlib.Path(src).read_bytes()
    recs = _records(bytes(raw))
    it = iter(recs)
    ncell, nfull = (mp // 2) * (np_ // 2) * (lp // 2), mp * np_ * lp

    def take(dtype, count=None):
        try:
            b = next(it)
        except StopIteration:
            raise RadRestartError("the file ends early") from None
        a = np.frombuffer(b, dtype=dtype)
        if count is not None and a.size != count:
            raise RadRestartError(f"record of {a.size} values where {count} are expected")
        return a.copy()

    d = {}
    for k in ("qe", "qa", "ql"):
        d[k] = take("<f8", ncell).reshape(lp // 2, np_ // 2, mp // 2)
    d["wall_rad_T"] = take("<f8", nfull).reshape(lp, np_, mp)
    g = take("<f8")
    if g.size < 5:
        raise RadRestartError("short emission totals record")
    d.update(zip(TOTALS_G, g[:5].tolist()))
    d.update(zip(TOTALS_W, take("<f8", 5).tolist()))
    d.update(zip(TOTALS_S, take("<f8", 6).tolist()))
    d["q_melt"], d["q_wall_loss"] = take("<f8", 2).tolist()
    d["q_exhaust"], d["q_rad_inlet"], d["q_rad_outlet"] = take("<f8", 3).tolist()
    for k in COUNTS:
        d[k] = int(take("<i4", 1)[0])
    for k in SCALARS:
        d[k] = float(take("<f8", 1)[0])
    d["aoxid"], d["aform"] = take("<f8", 2).tolist()
    d["avg_wall_T"] = float(take("<f8", 1)[0])
    nb = d["b_cnt"]
    for k in PATCH_INT:
        d[k] = take("<i2", nb).astype(np.int32)
    for k in ("patch_area", "b_face_area"):
        d[k] = take("<f8", nb)
    if d["preset_vf"] == 1:
        d["vf"] = take("<f8", nb * nb).reshape(nb, nb, order="F")
        d["vf_sum"] = take("<f8", nb)
    for k in PATCH_REAL:
        d[k] = take("<f8", nb)
    for k in CENTRE_INT:
        d[k] = take("<i2", nb).astype(np.int32)
    return d


def collect(solver, rad: dict, wall: dict, *, q_exhaust: float = 0.0, svf_r: float = 0.0,
            qa_s0_prev: float = 0.0) -> dict:
    """The content of the file RAD_EMIS writes after the handle's last volume
    transfer (`rad`, from rad_transfer) and wall exchange (`wall`, from
    wall_totals).  QRN1's totals of QA by cell kind (Qrn.f90:249-275) come
    from the transfer; the wall-emission totals QEW_*, QES0, QLS_G and QLS_A
    are zero as in the reference (Qrn.f90:571-600, Rad_emis.f90:136,
    Setup.f90:722-728); QA_S0/QA_S1 are the net radiation to the melt
    surface in MW and its change since `qa_s0_prev` (Qrn.f90:402-405);
    `q_exhaust` is EXTR's exhaust enthalpy flow of the iteration and
    `svf_r` MSFLOW's mean soot volume fraction."""
    case = solver.case
    f = solver.download()
    mp, np_, lp = case.mp, case.np, case.lp
    d = {"qe": f.arrays["qe"].copy(), "qa": f.arrays["qa"].copy(),
         "ql": np.zeros_like(f.arrays["qa"])}
    ints = {k: solver.wall_array(k).astype(np.int32) for k in PATCH_INT + CENTRE_INT}
    reals = {k: solver.wall_array(k.lower() if k == "b_T" else k) for k in PATCH_REAL + ("patch_area", "b_face_area")}
    # wall temperatures at the closed cell of each wall patch, in patch order
    # (Qwall.f90:1202-1208)
    wt = np.zeros((lp, np_, mp))
    for n in np.flatnonzero(ints["b_typ"] == 1):
        wt[ints["bc_k"][n] - 1, ints["bc_j"][n] - 1, ints["bc_i"][n] - 1] = reals["b_T"][n]
    d["wall_rad_T"] = wt
    d.update(qeg0=rad["qe_sum_from_open"], qeg_g=rad["qa_sum_to_open"], qeg_w=rad["qa_sum_to_wall"],
             qeg_s=rad["qa_sum_to_melt"], qeg_io=rad["qa_sum_to_inlet"] + rad["qa_sum_to_exit"])
    d.update({k: 0.0 for k in TOTALS_W}, qes0=0.0, qls_g=0.0, qls_a=0.0, svf_r=svf_r)
    g0 = (d["qeg_s"] + d["qew_s"] - d["qes0"]) * 1.0e-6
    d["qa_s1"], d["qa_s0"] = g0 - qa_s0_prev, g0
    d.update(q_melt=wall["q_melt"], q_wall_loss=wall["q_wall_loss"], q_exhaust=q_exhaust,
             q_rad_inlet=wall["q_rad_inlet"], q_rad_outlet=wall["q_rad_outlet"])
    typ, area = ints["b_typ"], reals["patch_area"]
    # the counts and area totals in patch order (Qwall.f90:733-748)
    tot = {1: 0.0, 4: 0.0, 2: 0.0, 3: 0.0}
    for t, a in zip(typ.tolist(), area.tolist()):
        key = t if t in (1, 4, 2) else 3
        tot[key] = tot[key] + a
    d.update(b_cnt=int(typ.size), preset_vf=1, iterw=int(wall["sweeps"]),
             iwall_count=int((typ == 1).sum()), imelt_count=int((typ == 4).sum()),
             inlet_count=int((typ == 2).sum()), iexit_count=int(((typ != 1) & (typ != 4) & (typ != 2)).sum()),
             wall_area_total=tot[1], melt_area_total=tot[4], inlet_area_total=tot[2], exit_area_total=tot[3],
             boundary_area_total=((tot[1] + tot[4]) + tot[2]) + tot[3])
    for k in ("q_incident_total", "q_incident_wall", "q_incident_inlet", "q_incident_exit", "q_incident_melt",
              "qconv_total", "avg_wall_T"):
        d[k] = wall[k]
    d["aoxid"], d["aform"] = case.params.aoxid, case.params.aform
    d.update(ints)
    d.update(reals)
    d["vf"] = solver.wall_vf()
    d["vf_sum"] = solver.wall_array("vf_sum")
    return d


def restore(solver, d: dict) -> None:
    """Gives a handle whose wall exchange is set up the wall state of the
    file (rad_emis_rr): the patch radiosities and temperatures the next
    exchange starts from, the sweep counter, the melt heat flux its outer
    loop compares against and the mean wall temperature.  The patch list of
    the file must be the handle's."""
    for k in ("b_typ", "b_i", "b_j", "b_k", "b_orient", "b_direct"):
        mine = solver.wall_array(k).astype(np.int32)
        if mine.size != d["b_cnt"] or not np.array_equal(mine, np.asarray(d[k], dtype=np.int32)):
            raise RadRestartError(f"the file's boundary patches differ from the case's ({k})")
    for k in ("radiosity", "b_T"):
        v = np.asarray(d[k], dtype=np.float64)
        if not np.all(np.isfinite(v)):
            raise RadRestartError(f"non-finite {k}")
        solver.wall_put(k.lower(), v)
    solver.wall_put("iterw", float(d["iterw"]))
    solver.wall_put("q_melt", float(d["q_melt"]))
    if not math.isfinite(d["avg_wall_T"]):
        raise RadRestartError("non-finite avg_wall_T")
    solver.wall_put("avg_wall_T", float(d["avg_wall_T"]))
