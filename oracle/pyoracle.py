"""ctypes wrapper of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module, as the checker; the product never imports it.
"""
from __future__ import annotations

import ctypes as C
import pathlib
import sys

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

from gfm_gb300 import abi  # noqa: E402
from gfm_gb300.solver import Case, Fields  # noqa: E402

from . import build as _build  # noqa: E402

STEP_WALLFN, STEP_MOMASM, STEP_PSOLVE, STEP_MOMSOLVE, STEP_PCORR, STEP_VELCORR, STEP_GSLV3V, STEP_SCALARS, STEP_PROPS, STEP_ALL = range(1, 11)

_lib = None


def load(check_bounds: bool = False) -> C.CDLL:
    global _lib
    if _lib is not None and not check_bounds:
        return _lib
    lib = C.CDLL(str(_build.build(check_bounds=check_bounds)))
    dp = C.POINTER(C.c_double)
    lib.gfo_create.restype = C.c_void_p
    lib.gfo_create.argtypes = [C.POINTER(abi.GfmGrid), C.POINTER(abi.GfmParams), C.POINTER(abi.GfmFields)]
    lib.gfo_destroy.argtypes = [C.c_void_p]
    lib.gfo_initsv.argtypes = [C.c_void_p]
    lib.gfo_gflow.argtypes = [C.c_void_p, C.c_int, C.POINTER(abi.GfmIterStats), C.POINTER(C.c_int)]
    lib.gfo_gflow_steps.argtypes = [C.c_void_p, C.c_int]
    lib.gfo_download.argtypes = [C.c_void_p, C.POINTER(abi.GfmFields)]
    lib.gfo_get_array.restype = C.c_long
    lib.gfo_get_array.argtypes = [C.c_void_p, C.c_char_p, dp, C.c_long]
    lib.gfo_adlbl3.argtypes = [C.c_void_p, dp, dp, C.POINTER(dp), dp] + [C.c_int] * 7
    lib.gfo_calc_residual.restype = C.c_double
    lib.gfo_calc_residual.argtypes = [C.c_void_p, dp, dp, C.POINTER(dp), dp] + [C.c_int] * 6
    lib.gfo_rad_transfer.argtypes = [C.c_void_p, C.POINTER(abi.GfmRadTotals)]
    lib.gfo_wall_setup.argtypes = [C.c_void_p, C.POINTER(abi.GfmWallSpec)]
    lib.gfo_wall_patch_list.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.c_int]
    lib.gfo_wall_totals.argtypes = [C.c_void_p, C.POINTER(abi.GfmWallTotals)]
    lib.gfo_minor_set.argtypes = [C.c_void_p, C.POINTER(abi.GfmMinor)]
    lib.gfo_minor_get.argtypes = [C.c_void_p, C.POINTER(abi.GfmMinor)]
    lib.gfo_rad_emission.argtypes = [C.c_void_p]
    lib.gfo_initsvm.argtypes = [C.c_void_p, C.c_int]
    lib.gfo_msflow.argtypes = [C.c_void_p, C.c_int, C.POINTER(abi.GfmMsflowStats)]
    for n in ("gfo_da", "gfo_tgamf", "gfo_emf", "gfo_rif3", "gfo_t_to_enth", "gfo_enth_to_t", "gfo_zy1", "gfo_atand"):
        getattr(lib, n).restype = C.c_double
    lib.gfo_da.argtypes = [C.c_double, C.c_double]
    lib.gfo_tgamf.argtypes = [C.c_double]
    lib.gfo_emf.argtypes = [C.c_double, C.c_double]
    lib.gfo_atand.argtypes = [C.c_double]
    lib.gfo_rif3.argtypes = [C.c_double]
    lib.gfo_zy1.argtypes = [dp, dp, C.c_double, C.c_int]
    lib.gfo_t_to_enth.argtypes = [dp, C.c_double]
    lib.gfo_enth_to_t.argtypes = [dp, C.c_double, C.c_double]
    lib.gfo_conc.argtypes = [dp]
    lib.gfo_case_build.argtypes = [C.POINTER(abi.GfmCaseSpec), C.c_char_p, C.POINTER(abi.GfmCase)]
    lib.gfo_case_free.argtypes = [C.POINTER(abi.GfmCase)]
    if not check_bounds:
        _lib = lib
    return lib


class OracleCase(Case):
    """A synthetic furnace built by the oracle's own start-up (gfo_case_build:
    GRID3, SETUP, SBC, gen_initial_guess, wall patches, kinetics table) in
    place of the product's gfm_case_build; the same interface as Case, and
    nothing of the product library is loaded."""

    def __init__(self, cfg, check_bounds: bool = False):
        self.cfg = cfg
        self.lib = load(check_bounds)
        self.c = abi.GfmCase()
        self.summary = None
        self.name = cfg.name
        self.spec = cfg.to_spec()
        rc = self.lib.gfo_case_build(C.byref(self.spec), str(abi.KINETIC_PATH).encode(), C.byref(self.c))
        if rc != 0:
            raise RuntimeError(f"gfo_case_build: {rc}")
        self._dims()

    def close(self) -> None:
        if self.c.priv:
            self.lib.gfo_case_free(C.byref(self.c))


class Oracle:
    """FP64 restatement of GFLOW/SPHASE on one case's host state."""

    def __init__(self, case: Case, fields: Fields | None = None, check_bounds: bool = False,
                 adi_mode: int | None = None):
        """adi_mode: plane order of the line solves (abi.GFM_ADI_MARCH, the
        reference's, or abi.GFM_ADI_REDBLACK, the GPU production order); None
        keeps the case's."""
        self.lib = load(check_bounds)
        self.case = case
        fld = fields if fields is not None else case.initial_fields()
        f = fld.to_c()   # pointers into fld's arrays: fld must outlive the call
        prm = abi.GfmParams.from_buffer_copy(case.params)
        if adi_mode is not None:
            prm.adi_mode = adi_mode
        self.o = self.lib.gfo_create(C.byref(case.grid), C.byref(prm), C.byref(f))
        del fld
        if not self.o:
            raise RuntimeError("gfo_create failed")

    def initsv(self) -> None:
        self.lib.gfo_initsv(self.o)

    def gflow(self, n: int = 1) -> tuple[dict, int]:
        st = abi.GfmIterStats()
        nd = C.c_int(0)
        self.lib.gfo_gflow(self.o, n, C.byref(st), C.byref(nd))
        return st.as_dict(), nd.value

    def gflow_steps(self, stop_after: int) -> None:
        self.lib.gfo_gflow_steps(self.o, stop_after)

    def rad_transfer(self) -> dict:
        """Volume radiation transfer from the current T; QE and QA are replaced."""
        t = abi.GfmRadTotals()
        rc = self.lib.gfo_rad_transfer(self.o, C.byref(t))
        if rc != 0:
            raise RuntimeError(f"gfo_rad_transfer: {rc}")
        return t.as_dict()

    def wall_setup(self, spec=None) -> None:
        """Turns on the wall radiosity exchange at the end of rad_transfer,
        with the case's wall inputs unless `spec` is given."""
        spec = spec if spec is not None else self.case.c.wall
        rc = self.lib.gfo_wall_setup(self.o, C.byref(spec))
        if rc != 0:
            raise RuntimeError(f"gfo_wall_setup: {rc}")

    def wall_patch_list(self) -> np.ndarray:
        n = self.lib.gfo_wall_patch_list(self.o, None, 0)
        out = np.zeros(6 * n, dtype=np.int32)
        self.lib.gfo_wall_patch_list(self.o, out.ctypes.data_as(C.POINTER(C.c_int)), n)
        return out.reshape(n, 6)

    def wall_totals(self) -> dict:
        t = abi.GfmWallTotals()
        rc = self.lib.gfo_wall_totals(self.o, C.byref(t))
        if rc != 0:
            raise RuntimeError(f"gfo_wall_totals: {rc}")
        return t.as_dict()

    def patch_array(self, name: str) -> np.ndarray:
        out = np.zeros(self.case.grid.b_cnt)
        got = self.lib.gfo_get_array(self.o, name.encode(), abi.dptr(out), out.size)
        if got != out.size:
            raise KeyError(name)
        return out

    def rad_emission(self) -> None:
        """The emission-only source QE from the current T (rad_qe_only)."""
        rc = self.lib.gfo_rad_emission(self.o)
        if rc != 0:
            raise RuntimeError(f"gfo_rad_emission: {rc}")

    def initsvm(self, restart: bool = False) -> None:
        rc = self.lib.gfo_initsvm(self.o, int(restart))
        if rc != 0:
            raise RuntimeError(f"gfo_initsvm: {rc}")

    def msflow(self, maxms: int) -> dict:
        st = abi.GfmMsflowStats()
        rc = self.lib.gfo_msflow(self.o, maxms, C.byref(st))
        if rc != 0:
            raise RuntimeError(f"gfo_msflow: {rc}")
        return st.as_dict()

    def minor_set(self, m) -> None:
        """The minor species state (a gfm_gb300.solver.Minor) the band model
        and MSFLOW work on."""
        rc = self.lib.gfo_minor_set(self.o, C.byref(m.to_c()))
        if rc != 0:
            raise RuntimeError(f"gfo_minor_set: {rc}")

    def minor_get(self):
        from gfm_gb300.solver import Minor
        out = Minor.empty(self.case.mp, self.case.np, self.case.lp)
        c = out.to_c()
        rc = self.lib.gfo_minor_get(self.o, C.byref(c))
        if rc != 0:
            raise RuntimeError(f"gfo_minor_get: {rc}")
        out.update_scalars(c)
        return out

    def download(self) -> Fields:
        out = Fields.empty(self.case.mp, self.case.np, self.case.lp)
        f = out.to_c()
        self.lib.gfo_download(self.o, C.byref(f))
        out.update_scalars(f)
        return out

    def array(self, name: str) -> np.ndarray:
        n = self.case.mp * self.case.np * self.case.lp
        out = np.zeros(n)
        got = self.lib.gfo_get_array(self.o, name.encode(), abi.dptr(out), n)
        if got != n:
            raise KeyError(name)
        return out.reshape(self.case.lp, self.case.np, self.case.mp)

    def close(self) -> None:
        if self.o:
            self.lib.gfo_destroy(self.o)
            self.o = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
