"""The GPU path on the reference's own cases (tests/golden): TC21 case 0041
read from its gd/sbc/it/relaxfactor files (fresh start) and from its
converged restart file, the other shipped cases from their files, against
the oracle on the same inputs and against the reference's logs of the fresh
starts.  Tolerances as in test_gpu_parity: 1e-9 relative L2 per field for
FP64 in the reference plane order, 1e-4 for the mixed form."""
import lzma
import shutil

import numpy as np
import pytest

from gfm_gb300 import Case, GpuSolver, abi
from oracle.pyoracle import Oracle

from .test_case_files import CASES, GOLD, INPUTS, case_inputs, check_against_log, half_blocked_dir, read_case
from .test_gpu_parity import FP64_TOL, MIXED_TOL, field_errors

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def case_dir(tmp_path_factory):
    d = tmp_path_factory.mktemp("case0041_gpu")
    for n in INPUTS:
        shutil.copyfile(GOLD / n, d / n)
    (d / "rg0041c.d").write_bytes(lzma.decompress((GOLD / "rg0041c.d.xz").read_bytes()))
    return d


def pair(case, n, adi=abi.GFM_ADI_MARCH, prec=abi.GFM_PREC_FP64):
    g = GpuSolver(case, adi_mode=adi, precision=prec)
    g.start()
    o = Oracle(case, adi_mode=adi)
    o.initsv()
    sg = [g.gflow(1)[0] for _ in range(n)]
    so = [o.gflow(1)[0] for _ in range(n)]
    fg, fo = g.download(), o.download()
    g.close()
    o.close()
    return sg, so, fg, fo, case.ibcell() <= 0


def test_fresh_start_fp64_matches_oracle(case_dir):
    case = Case.from_files(case_dir, "0041")
    sg, so, fg, fo, mask = pair(case, 2)
    err = field_errors(fg, fo, mask)
    assert max(err.values()) < FP64_TOL, err
    for a, b in zip(sg, so):
        for k in ("res_mass", "res_mass_max", "p_resid", "gfex", "factor", "tave", "tmean_ex"):
            assert a[k] == pytest.approx(b[k], rel=FP64_TOL, abs=1e-300), k


@pytest.mark.parametrize("num", ("0040", "1207"))
def test_other_cases_fp64_match_oracle(num, tmp_path):
    """Case 0040 (another port and flue layout) and case 1207 (y-direction
    inlet blocks, a 77-cell long furnace): two FP64 iterations."""
    case = read_case(num, tmp_path)
    sg, so, fg, fo, mask = pair(case, 2)
    err = field_errors(fg, fo, mask)
    assert max(err.values()) < FP64_TOL, err
    assert sg[-1]["res_mass"] == pytest.approx(so[-1]["res_mass"], rel=FP64_TOL)


@pytest.mark.parametrize("num", CASES)
def test_gpu_follows_the_reference_log_of_the_fresh_start(num, tmp_path):
    g = GpuSolver(read_case(num, tmp_path), adi_mode=abi.GFM_ADI_MARCH, precision=abi.GFM_PREC_FP64)
    g.start()
    stats = [g.gflow(1)[0] for _ in range(40)]
    g.close()
    check_against_log(num, stats)


def test_fresh_start_mixed_matches_oracle(case_dir):
    """Mixed precision in the reference's plane order after 3 iterations.
    Every field but the velocities stays within MIXED_TOL.  The velocities of
    this case (78 m/s angled fuel jets) differ from the oracle by 1.1e-4 to
    2.5e-4 relative L2 (measured), which is bounded at 5e-4.  That gap is the
    mixed path's FP32 arithmetic, not the rounding of its inputs: the FP64
    path started from the fresh-start fields rounded to FP32 stays within
    1e-6 of the oracle (measured 4e-8), which the test checks as well.  An
    FP32 exponential-scheme weight through expm1f and an FP64 per-cell mass
    imbalance were both tried and moved the velocity errors by no more than
    their spread (1.3e-4 to 6.0e-4)."""
    case = Case.from_files(case_dir, "0041")
    sg, so, fg, fo, mask = pair(case, 3, abi.GFM_ADI_MARCH, abi.GFM_PREC_MIXED)
    err = field_errors(fg, fo, mask)
    # the FP64 path from FP32-rounded inputs, against the oracle
    g = GpuSolver(case, adi_mode=abi.GFM_ADI_MARCH, precision=abi.GFM_PREC_FP64)
    f = case.initial_fields()
    for k, a in f.arrays.items():
        f.arrays[k] = a.astype(np.float32).astype(np.float64)
    g.upload(f)
    g.initsv()
    for _ in range(3):
        g.gflow(1)
    fr = g.download()
    g.close()
    sens = field_errors(fr, fo, mask)
    msg = " ".join(f"{k}={v:.3e}/{sens[k]:.3e}" for k, v in err.items())
    assert max(v for k, v in err.items() if k not in ("u", "v", "w")) < MIXED_TOL, msg
    assert max(sens.values()) < 1e-6, msg
    assert max(err["u"], err["v"], err["w"]) < 5e-4, msg
    assert sg[-1]["res_mass"] == pytest.approx(so[-1]["res_mass"], rel=1e-3)


@pytest.mark.parametrize("prec,tol", [(abi.GFM_PREC_FP64, FP64_TOL), (abi.GFM_PREC_MIXED, MIXED_TOL)])
def test_fresh_start_redblack_matches_the_redblack_oracle(case_dir, prec, tol):
    """The benchmarked line order (red-black planes) against the oracle run in
    the same plane order: one iteration of TC21 case 0041 from its files,
    FP64 within 1e-9 and the mixed form within 1e-4 relative L2 per field."""
    case = Case.from_files(case_dir, "0041")
    sg, so, fg, fo, mask = pair(case, 1, abi.GFM_ADI_REDBLACK, prec)
    err = field_errors(fg, fo, mask)
    msg = " ".join(f"{k}={v:.3e}" for k, v in err.items())
    assert max(err.values()) < tol, msg
    assert sg[-1]["res_mass"] == pytest.approx(so[-1]["res_mass"], rel=tol * 10)


def test_redblack_mixed_converges_like_the_reference_log(case_dir):
    """The red-black line order is not the reference's, so its iterates are
    not compared cell by cell; its mass residual history on this case stays
    near the reference's logged one."""
    _, _, ref = case_inputs("0041")
    case = Case.from_files(case_dir, "0041")
    g = GpuSolver(case, adi_mode=abi.GFM_ADI_REDBLACK, precision=abi.GFM_PREC_MIXED)
    g.start()
    stats = [g.gflow(1)[0] for _ in range(40)]
    f = g.download()
    g.close()
    assert all(np.isfinite(a).all() for a in f.arrays.values())
    for it in (10, 20, 40):
        assert stats[it - 1]["res_mass"] == pytest.approx(ref["res_mass"][it - 1], rel=0.25), (it, stats[it - 1]["res_mass"])


def test_restart_fp64_matches_oracle(case_dir):
    case = Case.from_files(case_dir, "0041", restart=True)
    sg, so, fg, fo, mask = pair(case, 2)
    err = field_errors(fg, fo, mask)
    assert max(err.values()) < FP64_TOL, err
    assert sg[0]["itr_gas"] == so[0]["itr_gas"] == 7541
    assert sg[-1]["res_mass"] == pytest.approx(so[-1]["res_mass"], rel=FP64_TOL)


_MARCH_RUN = r"""
import hashlib, lzma, pathlib, shutil, sys, tempfile
sys.path.insert(0, {root!r})
from gfm_gb300 import Case, GpuSolver, abi
gold = pathlib.Path({gold!r})
with tempfile.TemporaryDirectory() as d:
    for n in {inputs!r}:
        shutil.copyfile(gold / n, pathlib.Path(d) / n)
    case = Case.from_files(d, "0041")
h = hashlib.sha256()
for prec in (abi.GFM_PREC_FP64, abi.GFM_PREC_MIXED):
    g = GpuSolver(case, adi_mode=abi.GFM_ADI_MARCH, precision=prec)
    g.start()
    st, _ = g.gflow(2)
    f = g.download()
    g.close()
    for k in sorted(f.arrays):
        h.update(f.arrays[k].tobytes())
    h.update(repr(st["res_mass"]).encode())
print(h.hexdigest())
"""


def test_march_row_batches_give_the_same_bits():
    """The default march computes the pivots of each call once, loads a
    line's rows four at a time, keeps the plane's line scratch in shared
    memory and gives a plane's y-lines and z-lines their own warps;
    GFM_MARCH_LAYOUT=contiguous keeps thread t on lines t, t + blockDim, ..
    of both kinds; GFM_MARCH_ROWS=1 runs the reference's row-by-row loop with
    field-sized scratch.  Two FP64 and two mixed iterations of TC21 give the
    same bits all three ways (each run is its own process: the variables are
    read once)."""
    import os
    import pathlib
    import subprocess
    import sys
    root = str(pathlib.Path(__file__).resolve().parents[1])
    code = _MARCH_RUN.format(root=root, gold=str(GOLD), inputs=INPUTS)
    out = []
    for rows, layout in (("4", "split"), ("4", "contiguous"), ("1", "contiguous")):
        env = dict(os.environ, GFM_MARCH_ROWS=rows, GFM_MARCH_LAYOUT=layout)
        r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr
        out.append(r.stdout.strip().splitlines()[-1])
    assert out[0] == out[1] == out[2]


@pytest.mark.parametrize("num", ("0041", "1207"))
def test_rad_transfer_matches_oracle_on_reference_cases(num, tmp_path):
    """The volume radiation transfer on the reference's own geometries (ports,
    a side flue, a stepped crown, a melt surface), gray kappa 0.5 1/m in every
    band, from the state after 3 FP64 iterations; tolerances of test_gpu_rad.
    Their obstacles make interior columns and the emitter's own column reach
    wall-corner splits (TC21: about 460k and 8.8k per transfer), which the
    kernel lists and adds in the reference's column order."""
    from .test_gpu_rad import _compare
    case = read_case(num, tmp_path, kappa=[0.5] * 16)
    o = Oracle(case)
    o.initsv()
    o.gflow(3)
    g = GpuSolver(case, precision=abi.GFM_PREC_FP64)
    g.upload(o.download())
    tg = g.rad_transfer()
    to = o.rad_transfer()
    _compare(g.download(), o.download(), tg, to)
    g.close()
    o.close()


def test_restart_with_emission_and_wall_sink_fp64_matches_oracle(case_dir):
    """From the converged restart (itr_gas 7540) with the emission-only
    radiation source and the fixed-temperature wall sink on (melt-surface
    patches at the melt temperature): 12 FP64 iterations, one emission update
    at the tenth, against the oracle."""
    case = Case.from_files(case_dir, "0041", restart=True, rad_emission=True, wall_sink=True, kappa=[0.5] * 16)
    sg, so, fg, fo, mask = pair(case, 12)
    err = field_errors(fg, fo, mask)
    assert max(err.values()) < FP64_TOL, err
    assert fg.i1st_rad_qe_done == fo.i1st_rad_qe_done == 1
    qe_g, qe_o = fg.arrays["qe"], fo.arrays["qe"]
    assert np.count_nonzero(qe_o) > 0
    assert np.linalg.norm(qe_g - qe_o) / np.linalg.norm(qe_o) < FP64_TOL
    for a, b in zip(sg, so):
        assert a["q_conv_total"] == pytest.approx(b["q_conv_total"], rel=FP64_TOL)


@pytest.mark.parametrize("adi,prec,n,tol", [(abi.GFM_ADI_MARCH, abi.GFM_PREC_FP64, 2, FP64_TOL),
                                            (abi.GFM_ADI_REDBLACK, abi.GFM_PREC_FP64, 2, FP64_TOL),
                                            (abi.GFM_ADI_REDBLACK, abi.GFM_PREC_MIXED, 1, MIXED_TOL)])
def test_half_blocked_cells_match_oracle(case_dir, tmp_path, adi, prec, n, tol):
    """TC21 case 0041 with half-blocked cells (IBCELL -1 and -2) and
    non-unit &GRD factors: VOL_C0 and AREA_C scale by BV_F and BA_F
    (Grid3.f90:395-471), the momentum volumes subtract the half cells
    (Gslv3x.f90:273-282).  GPU against the oracle in the same plane order."""
    case = Case.from_files(half_blocked_dir(case_dir, tmp_path / "half"), "0041")
    sg, so, fg, fo, mask = pair(case, n, adi, prec)
    err = field_errors(fg, fo, mask)
    msg = " ".join(f"{k}={v:.3e}" for k, v in err.items())
    assert max(err.values()) < tol, msg
    assert sg[-1]["res_mass"] == pytest.approx(so[-1]["res_mass"], rel=tol * 10)

