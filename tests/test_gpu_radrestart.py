"""A restart through the radiation restart on the GPU: a run of TC21 case
0041 (band model, wall exchange) writes rg and rr after a radiation call; a
new handle started from them, with the wall state restored, gives the next
radiation call the continuing run gives (Initsv.f90:312, Rad_emis.f90:17-110)."""
import numpy as np
import pytest

from gfm_gb300 import Case, GpuSolver, abi, radrestart

from .test_oracle_gas import converged, converged_dir

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def test_restart_from_rr_continues_the_run(tmp_path):
    case, minor = converged("0041", tmp_path, wall_sink=True)
    d = converged_dir("0041", tmp_path)
    a = GpuSolver(case, precision=abi.GFM_PREC_FP64)
    a.start()
    a.minor_upload(minor)
    a.wall_setup()
    rr = radrestart.collect(a, a.rad_transfer(), a.wall_totals())
    assert rr["b_cnt"] == case.grid.b_cnt and rr["iwall_count"] > 0 and rr["imelt_count"] > 0
    assert np.allclose(rr["vf"].sum(axis=1)[rr["vf_sum"] > 0], 1.0, atol=1e-12)
    case.write_restart(d / "rg0041c.d", a.download())
    radrestart.write(d / "rr0041c.d", rr)
    back = radrestart.read(d / "rr0041c.d", case.mp, case.np, case.lp)
    assert np.array_equal(back["radiosity"], rr["radiosity"]) and np.array_equal(back["vf"], rr["vf"])
    rad2 = a.rad_transfer()
    wall2 = a.wall_totals()

    c2 = Case.from_files(d, "0041", restart=True, gas_model=True, wall_sink=True, rad_restart=True)
    f2 = c2.initial_fields()
    assert np.array_equal(f2.arrays["qa"], rr["qa"]) and np.array_equal(f2.arrays["qe"], rr["qe"])
    b = GpuSolver(c2, precision=abi.GFM_PREC_FP64)
    b.start()
    b.minor_upload(minor)
    b.wall_setup()
    radrestart.restore(b, back)
    assert np.array_equal(b.wall_array("b_t"), rr["b_T"])
    rad2b = b.rad_transfer()
    wall2b = b.wall_totals()
    for k in rad2:
        assert rad2b[k] == pytest.approx(rad2[k], rel=1e-9, abs=1e-12), k
    # A restart is not the continuing run to the last bit, in the reference
    # either: the case read applies melt_surf_T again (relaxed against the
    # stored T_surf_prev) and INITSV interpolates the faces the wall exchange
    # had set.  The next exchange agrees to about 3e-7; the net radiation
    # through the inlets and exits, a difference of large terms, differs by
    # about 1e-6 of the incident total (2e-5 of itself).  The wall state
    # itself is restored exactly (the next test).
    scale = 1e-5 * wall2["q_incident_total"]
    for k in ("avg_wall_T", "q_melt", "q_wall_loss", "q_incident_total", "qconv_total", "q_rad_inlet",
              "q_rad_outlet"):
        assert wall2b[k] == pytest.approx(wall2[k], rel=1e-5, abs=scale), k
    # per patch the wall temperatures differ by up to 2.4e-5 of the largest
    for n in ("b_t", "radiosity"):
        assert _rel(b.wall_array(n), a.wall_array(n)) < 1e-4, n
    assert _rel(b.download().arrays["qa"], a.download().arrays["qa"]) < 1e-9


def test_restored_wall_state_continues_the_exchange_exactly(tmp_path):
    """The wall state alone: a handle given the continuing run's fields and
    the file's wall state makes the continuing run's next exchange."""
    case, minor = converged("0041", tmp_path, wall_sink=True)
    a = GpuSolver(case, precision=abi.GFM_PREC_FP64)
    a.start()
    a.minor_upload(minor)
    a.wall_setup()
    rr = radrestart.collect(a, a.rad_transfer(), a.wall_totals())
    fa = a.download()
    rad2, wall2 = a.rad_transfer(), a.wall_totals()
    b = GpuSolver(case, precision=abi.GFM_PREC_FP64)
    b.upload(fa)
    b.minor_upload(minor)
    b.wall_setup()
    radrestart.restore(b, rr)
    rad2b, wall2b = b.rad_transfer(), b.wall_totals()
    for k in rad2:
        assert rad2b[k] == pytest.approx(rad2[k], rel=1e-12, abs=1e-12), k
    for k in wall2:
        assert wall2b[k] == pytest.approx(wall2[k], rel=1e-12, abs=1e-12), k
    for n in ("b_t", "radiosity", "qrs"):
        assert _rel(b.wall_array(n), a.wall_array(n)) < 1e-12, n


def test_restore_refuses_another_patch_list(tmp_path):
    case, minor = converged("0041", tmp_path, wall_sink=True)
    a = GpuSolver(case, precision=abi.GFM_PREC_FP64)
    a.start()
    a.minor_upload(minor)
    a.wall_setup()
    rr = radrestart.collect(a, a.rad_transfer(), a.wall_totals())
    rr["b_i"] = rr["b_i"].copy()
    rr["b_i"][0] += 2
    with pytest.raises(radrestart.RadRestartError):
        radrestart.restore(a, rr)


def test_view_factors_of_the_mixed_path(tmp_path):
    """The mixed path keeps the view factors in FP32; gfm_gpu_wall_vf hands
    them out as doubles, row by row as the FP64 path does."""
    case, _ = converged("0041", tmp_path, wall_sink=True)
    out = {}
    for prec in (abi.GFM_PREC_FP64, abi.GFM_PREC_MIXED):
        g = GpuSolver(case, precision=prec)
        g.start()
        g.wall_setup()
        out[prec] = (g.wall_vf(), g.wall_array("vf_sum"))
    (v64, s64), (v32, s32) = out[abi.GFM_PREC_FP64], out[abi.GFM_PREC_MIXED]
    assert np.array_equal(s32, s64)
    assert np.array_equal(v32, v64.astype(np.float32).astype(np.float64))
