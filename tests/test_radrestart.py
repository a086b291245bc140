"""The radiation restart rr####c.d (Rad_emis.f90:17-110, 289-350): the
record layout of RAD_EMIS's writer, the round trip through rad_emis_rr's
reader, and the case restart that takes QE, QA and the wall temperatures
from it.  The shipped cases hold no rr files, so the layout is checked
against the reference's READ and WRITE statements record by record."""
import struct

import numpy as np
import pytest

from gfm_gb300 import radrestart

from .test_oracle_gas import converged, converged_dir


def _synthetic(mp, np_, lp, nb, preset_vf=1, seed=3):
    rng = np.random.default_rng(seed)
    cells = (lp // 2, np_ // 2, mp // 2)
    d = {k: rng.random(cells) for k in ("qe", "qa", "ql")}
    d["wall_rad_T"] = rng.random((lp, np_, mp))
    for k in radrestart.TOTALS_G + radrestart.TOTALS_W + radrestart.TOTALS_S:
        d[k] = float(rng.random())
    for k in ("q_melt", "q_wall_loss", "q_exhaust", "q_rad_inlet", "q_rad_outlet", "aoxid", "aform", "avg_wall_T"):
        d[k] = float(rng.random())
    for k in radrestart.SCALARS:
        d[k] = float(rng.random())
    d.update(b_cnt=nb, preset_vf=preset_vf, iterw=17, iwall_count=nb - 3, imelt_count=1, inlet_count=1,
             iexit_count=1)
    for k in radrestart.PATCH_INT + radrestart.CENTRE_INT:
        d[k] = rng.integers(-3, 300, nb).astype(np.int32)
    for k in radrestart.PATCH_REAL + ("patch_area", "b_face_area", "vf_sum"):
        d[k] = rng.random(nb)
    d["vf"] = rng.random((nb, nb))
    return d


@pytest.mark.parametrize("preset_vf", [1, 0])
def test_round_trip_and_record_layout(tmp_path, preset_vf):
    mp, np_, lp, nb = 10, 8, 6, 7
    d = _synthetic(mp, np_, lp, nb, preset_vf)
    p = tmp_path / "rr0001c.d"
    radrestart.write(p, d)
    raw = p.read_bytes()
    sizes = [len(r) for r in radrestart._records(raw)]
    nc, nf = (mp // 2) * (np_ // 2) * (lp // 2), mp * np_ * lp
    # RAD_EMIS's WRITE statements, in order (Rad_emis.f90:293-350)
    want = [8 * nc] * 3 + [8 * nf, 48, 40, 48, 16, 24] + [4] * 7 + [8] * 11 + [16, 8] + [2 * nb] * 6 + [8 * nb] * 2
    want += ([8 * nb * nb, 8 * nb] if preset_vf == 1 else []) + [8 * nb] * 7 + [2 * nb] * 4
    assert sizes == want
    back = radrestart.read(raw, mp, np_, lp)
    for k, v in d.items():
        if k == "vf" and preset_vf != 1:
            assert "vf" not in back
            continue
        if k == "vf_sum" and preset_vf != 1:
            continue
        if isinstance(v, np.ndarray):
            assert np.array_equal(np.asarray(back[k]), v), k
        else:
            assert back[k] == v, k
    # vf(n,m) is stored with n fastest: the second value is vf(2,1)
    if preset_vf == 1:
        vf_at = sum(sizes[:37]) + 8 * 37 + 4   # 37 records before vf
        assert struct.unpack_from("<d", raw, vf_at + 8)[0] == d["vf"][1, 0]
    # writing what was read gives the same bytes
    radrestart.write(tmp_path / "again.d", back)
    assert (tmp_path / "again.d").read_bytes() == raw


def test_five_value_emission_record_is_read(tmp_path):
    """rad_emis_rr reads five values from the record RAD_EMIS writes with six."""
    mp, np_, lp, nb = 6, 6, 6, 3
    d = _synthetic(mp, np_, lp, nb)
    raw = bytearray()
    recs = radrestart._records((lambda p: (radrestart.write(p, d), p.read_bytes())[1])(tmp_path / "a.d"))
    recs[4] = recs[4][:40]
    for r in recs:
        raw += radrestart._rec(r)
    back = radrestart.read(bytes(raw), mp, np_, lp)
    assert back["qeg_io"] == d["qeg_io"] and back["qes0"] == d["qes0"]


def test_truncated_or_foreign_file_is_refused(tmp_path):
    mp, np_, lp, nb = 6, 6, 6, 3
    p = tmp_path / "rr.d"
    radrestart.write(p, _synthetic(mp, np_, lp, nb))
    raw = p.read_bytes()
    with pytest.raises(radrestart.RadRestartError):
        radrestart.read(raw[:-5], mp, np_, lp)
    with pytest.raises(radrestart.RadRestartError):
        radrestart.read(raw, mp + 2, np_, lp)
    cut = radrestart._records(raw)[:20]
    with pytest.raises(radrestart.RadRestartError):
        radrestart.read(b"".join(radrestart._rec(r) for r in cut), mp, np_, lp)


def test_case_restart_takes_qe_qa_and_wall_temperatures(tmp_path):
    """rad_emis_rr after read_restart_data: QE and QA from the file, and the
    wall cell centres the file gives a temperature take it, with their
    enthalpy (Rad_emis.f90:91-100); every other cell keeps the gas restart's
    values."""
    case, _ = converged("0041", tmp_path)
    d = converged_dir("0041", tmp_path)
    f0 = case.initial_fields()
    mp, np_, lp = case.mp, case.np, case.lp
    ib = case.ibcell()
    walls = [(k, j, i) for k in range(1, lp, 2) for j in range(1, np_, 2) for i in range(1, mp, 2) if ib[k, j, i] == 1]
    assert len(walls) > 100
    rr = _synthetic(mp, np_, lp, 4)
    rr["wall_rad_T"] = np.zeros((lp, np_, mp))
    hot, cold = walls[::7], walls[3::7]
    for c in hot:
        rr["wall_rad_T"][c] = 1500.0
    for c in cold:
        rr["wall_rad_T"][c] = 900.0
    radrestart.write(d / "rr0041c.d", rr)
    from gfm_gb300 import Case
    c2 = Case.from_files(d, "0041", restart=True, gas_model=True, rad_restart=True)
    f2 = c2.initial_fields()
    assert np.array_equal(f2.arrays["qe"], rr["qe"]) and np.array_equal(f2.arrays["qa"], rr["qa"])
    t0 = case.params.t0
    h, species = 2, [0, 1, 5, 6, 8]   # GF's enthalpy and species components
    for c in hot:
        assert f2.arrays["t"][c] == 1500.0 / t0
    for c in cold:
        assert f2.arrays["t"][c] == 900.0 / t0
    gf0, gf2 = f0.arrays["gf"], f2.arrays["gf"]
    same = [(a, b) for a, b in zip(hot, cold) if np.array_equal(gf0[species][(slice(None),) + a],
                                                                gf0[species][(slice(None),) + b])]
    assert same and all(gf2[h][a] > gf2[h][b] for a, b in same)
    assert sum(gf2[h][c] != gf0[h][c] for c in hot + cold) > 0.9 * len(hot + cold)
    mask = np.ones(ib.shape, bool)
    for c in hot + cold:
        mask[c] = False
    assert np.array_equal(f2.arrays["t"][mask], f0.arrays["t"][mask])
    assert np.array_equal(f2.arrays["gf"][:, mask], f0.arrays["gf"][:, mask])
    with pytest.raises(ValueError):
        Case.from_files(d, "0041", restart=False, rad_restart=True)
    # a named file that is missing or too short is an error, as rad_emis_rr's
    # read errors stop the reference ("unable to read radiation restart file")
    from gfm_gb300.solver import GfmError
    with pytest.raises(GfmError):
        Case.from_files(d, "0041", restart=True, rad_restart=d / "rr9999c.d")
    (d / "short.d").write_bytes((d / "rr0041c.d").read_bytes()[:1000])
    with pytest.raises(GfmError):
        Case.from_files(d, "0041", restart=True, rad_restart=d / "short.d")
