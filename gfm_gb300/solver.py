"""Host-side mirror of the reference's solver interface over the C ABI.

``Case`` plays the role of the Fortran start-up (GRID3/SETUP/SBC/INITSV): it
builds the grid, the constants and the fresh-start fields in the reference's
doubled layout.  ``GpuSolver`` replaces ``CALL GFLOW`` (Sphase.f90:51) with
``gflow(n)``, keeps the reference's field layout at the boundary, and raises
``GfmError`` for every non-zero status, as the reference's ``stop_run`` ends
the run (A0main.f90:415-424).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import abi
from .configs import FurnaceCase


class GfmError(RuntimeError):
    def __init__(self, rc: int, msg: str):
        super().__init__(f"gfm status {rc}: {msg}")
        self.rc = rc


FIELD_NAMES = ("p", "t", "dnst", "theta", "tmu", "gama", "crate", "hrate", "bs_hprev")


@dataclass
class Fields:
    """Host fields in the reference layout: arrays of shape (LP,NP,MP) C-order
    = Fortran (MP,NP,LP); ug (3,LP,NP,MP); gf (9,LP,NP,MP); qa/qe (LZ,NZ,MZ)."""
    arrays: dict
    itr_gas: int = 0
    do_rad_qe_only_cnt: int = 0
    i1st_rad_qe_done: int = 0
    factor: float = 1.0
    fadj: float = 0.0
    gfin0: float = 0.0
    q_h_in: float = 0.0

    @staticmethod
    def empty(mp: int, np_: int, lp: int) -> "Fields":
        shp = (lp, np_, mp)
        arr = {n: np.zeros(shp) for n in FIELD_NAMES}
        arr["ug"] = np.zeros((3,) + shp)
        arr["gf"] = np.zeros((9,) + shp)
        arr["qa"] = np.zeros((lp // 2, np_ // 2, mp // 2))
        arr["qe"] = np.zeros((lp // 2, np_ // 2, mp // 2))
        return Fields(arr)

    def to_c(self) -> abi.GfmFields:
        f = abi.GfmFields()
        for n in FIELD_NAMES + ("ug", "gf", "qa", "qe"):
            a = self.arrays[n]
            assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
            setattr(f, n, abi.dptr(a))
        f.itr_gas, f.do_rad_qe_only_cnt, f.i1st_rad_qe_done = self.itr_gas, self.do_rad_qe_only_cnt, self.i1st_rad_qe_done
        f.factor, f.fadj, f.gfin0, f.q_h_in = self.factor, self.fadj, self.gfin0, self.q_h_in
        return f

    def update_scalars(self, f: abi.GfmFields) -> None:
        self.itr_gas, self.do_rad_qe_only_cnt, self.i1st_rad_qe_done = f.itr_gas, f.do_rad_qe_only_cnt, f.i1st_rad_qe_done
        self.factor, self.fadj, self.gfin0, self.q_h_in = f.factor, f.fadj, f.gfin0, f.q_h_in

    def copy(self) -> "Fields":
        return Fields({k: v.copy() for k, v in self.arrays.items()}, self.itr_gas, self.do_rad_qe_only_cnt,
                      self.i1st_rad_qe_done, self.factor, self.fadj, self.gfin0, self.q_h_in)


class Minor:
    """The minor species state of MSFLOW in the reference layout: gfm
    (7, LP, NP, MP) C-order views of GFM(MP,NP,LP,7), smf and the soot
    sources (LP, NP, MP), rrms (5, LZ, NZ, MZ)."""

    def __init__(self, gfm, smf, bs_soot_prev, sfp_soot_prev, rrms, itr_ms: int = 0, imscon: int = 0):
        self.gfm, self.smf, self.bs_soot_prev, self.sfp_soot_prev, self.rrms = gfm, smf, bs_soot_prev, sfp_soot_prev, rrms
        self.itr_ms, self.imscon = itr_ms, imscon
        self._c = None

    @staticmethod
    def empty(mp: int, np_: int, lp: int) -> "Minor":
        z = lambda *sh: np.zeros(sh, dtype=np.float64)
        return Minor(z(abi.NSP_MINOR, lp, np_, mp), z(lp, np_, mp), z(lp, np_, mp), z(lp, np_, mp),
                     z(5, lp // 2, np_ // 2, mp // 2))

    def to_c(self) -> abi.GfmMinor:
        for a in (self.gfm, self.smf, self.bs_soot_prev, self.sfp_soot_prev, self.rrms):
            assert a.flags.c_contiguous and a.dtype == np.float64
        p = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
        self._c = abi.GfmMinor(p(self.gfm), p(self.smf), p(self.bs_soot_prev), p(self.sfp_soot_prev), p(self.rrms),
                               int(self.itr_ms), int(self.imscon))
        return self._c

    def update_scalars(self, m: abi.GfmMinor) -> None:
        self.itr_ms, self.imscon = m.itr_ms, m.imscon

    def copy(self) -> "Minor":
        return Minor(self.gfm.copy(), self.smf.copy(), self.bs_soot_prev.copy(), self.sfp_soot_prev.copy(),
                     self.rrms.copy(), self.itr_ms, self.imscon)


class Case:
    """A built case (host arrays owned by the native library): a synthetic
    furnace (``Case(cfg)``) or a GFM case directory (``Case.from_files``)."""

    def __init__(self, cfg: FurnaceCase | None, lib: C.CDLL | None = None):
        self.cfg = cfg
        self.lib = lib or abi.load_library()
        self.c = abi.GfmCase()
        self.summary = None
        if cfg is None:
            return
        self.name = cfg.name
        self.spec = cfg.to_spec()
        rc = self.lib.gfm_case_build(C.byref(self.spec), str(abi.KINETIC_PATH).encode(), C.byref(self.c))
        if rc != abi.GFM_OK:
            raise GfmError(rc, "gfm_case_build failed")
        self._dims()

    def _dims(self) -> None:
        g = self.c.grid
        self.mp, self.np, self.lp = g.mp, g.np, g.lp
        self.ncells = g.ncells

    @classmethod
    def from_files(cls, case_dir, runum: str, relax=None, kinetic=None, restart: bool = False,
                   sigma_eps: float = 1.0, wall_sink: bool = False, t_wall_k: float = 1700.0,
                   rad_emission: bool = False, kappa=None, maxgi: int = 0,
                   adi_mode: int = abi.GFM_ADI_MARCH, precision: int = abi.GFM_PREC_FP64,
                   gas_model: bool = False, rad_restart=None, lib: C.CDLL | None = None) -> "Case":
        """The start-up the Fortran host does from a case directory: reads
        gd<runum>c.dat, sbc<runum>c.dat, it<runum>t.dat (when present),
        relaxfactorc.txt (``relax``, default: in the case directory) and the
        kinetics table, and with ``restart`` the restart file rg<runum>c.d
        (A0main.f90:158-190).  ``summary`` holds what GRID3/SBC derived.
        ``gas_model`` takes the absorption coefficients from RAD_GAS and
        SOOTA on the minor species instead of ``kappa``.  ``rad_restart``
        (with ``restart``): the radiation restart rr<runum>c.d to read after
        it, True for the one in the case directory or a path (rad_emis_rr,
        Rad_emis.f90:17-110; the wall state it holds goes to a handle with
        ``radrestart.restore``)."""
        import pathlib
        d = pathlib.Path(case_dir)
        it = d / f"it{runum}t.dat"
        paths = {
            "gd": d / f"gd{runum}c.dat", "sbc": d / f"sbc{runum}c.dat",
            "relax": pathlib.Path(relax) if relax else d / "relaxfactorc.txt",
            "it": it if it.exists() else None,
            "rg": d / f"rg{runum}c.d" if restart else None,
            "kinetic": pathlib.Path(kinetic) if kinetic else abi.KINETIC_PATH,
            "rr": None,
        }
        if rad_restart is not None and rad_restart is not False:
            if not restart:
                raise ValueError("a radiation restart is read after the gas restart (restart=True)")
            paths["rr"] = d / f"rr{runum}c.d" if rad_restart is True else pathlib.Path(rad_restart)
        self = cls(None, lib)
        self.name = f"case{runum}"
        self._paths = {k: (str(v).encode() if v is not None else None) for k, v in paths.items()}
        files = abi.GfmCaseFiles(**self._paths)
        opt = abi.GfmCaseOptions()
        opt.sigma_eps, opt.wall_sink, opt.t_wall_k, opt.rad_emission = sigma_eps, int(wall_sink), t_wall_k, int(rad_emission)
        for l, k in enumerate(kappa or []):
            opt.kappa[l] = k
        opt.maxgi, opt.adi_mode, opt.precision = maxgi, adi_mode, precision
        opt.gas_model = int(gas_model)
        summ = abi.GfmCaseSummary()
        rc = self.lib.gfm_case_read(C.byref(files), C.byref(opt), C.byref(self.c), C.byref(summ))
        if rc != abi.GFM_OK:
            raise GfmError(rc, f"gfm_case_read failed for {d} ({runum})")
        self.summary = summ.as_dict()
        self._dims()
        return self

    def read_minor(self, path) -> "Minor":
        """The minor species restart rs<runum>c.d (SAV3FM's records)."""
        m = Minor.empty(self.mp, self.np, self.lp)
        rc = self.lib.gfm_minor_read(str(path).encode(), C.byref(self.c.grid), C.byref(m.to_c()))
        if rc != abi.GFM_OK:
            raise GfmError(rc, f"gfm_minor_read failed for {path}")
        m.itr_ms = m._c.itr_ms
        return m

    def write_minor(self, path, m: "Minor") -> None:
        rc = self.lib.gfm_minor_write(str(path).encode(), C.byref(self.c.grid), C.byref(m.to_c()))
        if rc != abi.GFM_OK:
            raise GfmError(rc, f"gfm_minor_write failed for {path}")

    def t_surf_prev(self) -> np.ndarray:
        """T_surf_prev(MZ,NZ) (K) as an (NZ, MZ) C-order array."""
        t = self.c.tail
        return np.ctypeslib.as_array(t.t_surf_prev, shape=(t.mz * t.nz,)).reshape(t.nz, t.mz).copy()

    def write_restart(self, path, fields: "Fields | None" = None) -> None:
        """Writes rg####c.d (SAV3F layout, Sav3f.f90:21-88) of ``fields``
        (default: the case's own start-up fields) with this case's restart
        tail."""
        fld = fields if fields is not None else self.initial_fields()
        f = fld.to_c()
        rc = self.lib.gfm_restart_write(str(path).encode(), C.byref(self.c.grid), C.byref(f), C.byref(self.c.tail))
        if rc != abi.GFM_OK:
            raise GfmError(rc, f"gfm_restart_write failed for {path}")

    @property
    def grid(self) -> abi.GfmGrid:
        return self.c.grid

    @property
    def params(self) -> abi.GfmParams:
        return self.c.params

    def ibcell(self) -> np.ndarray:
        n = self.mp * self.np * self.lp
        return np.ctypeslib.as_array(self.c.grid.ibcell, shape=(n,)).reshape(self.lp, self.np, self.mp).copy()

    def initial_fields(self) -> Fields:
        """Copy of the fresh-start fields (before INITSV's interpolation)."""
        n = self.mp * self.np * self.lp
        nc = (self.mp // 2) * (self.np // 2) * (self.lp // 2)
        f = self.c.fields
        shp = (self.lp, self.np, self.mp)
        arr = {}
        for name in FIELD_NAMES:
            arr[name] = np.ctypeslib.as_array(getattr(f, name), shape=(n,)).reshape(shp).copy()
        arr["ug"] = np.ctypeslib.as_array(f.ug, shape=(3 * n,)).reshape((3,) + shp).copy()
        arr["gf"] = np.ctypeslib.as_array(f.gf, shape=(9 * n,)).reshape((9,) + shp).copy()
        csh = (self.lp // 2, self.np // 2, self.mp // 2)
        arr["qa"] = np.ctypeslib.as_array(f.qa, shape=(nc,)).reshape(csh).copy()
        arr["qe"] = np.ctypeslib.as_array(f.qe, shape=(nc,)).reshape(csh).copy()
        return Fields(arr, f.itr_gas, f.do_rad_qe_only_cnt, f.i1st_rad_qe_done, f.factor, f.fadj, f.gfin0, f.q_h_in)

    def close(self) -> None:
        if self.c.priv:
            self.lib.gfm_case_free(C.byref(self.c))

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def write_case_files(cfg: FurnaceCase, case_dir, runum: str, lib: C.CDLL | None = None) -> None:
    """Writes a synthetic furnace as a GFM case directory (gd/sbc/relaxfactorc
    files, gfm_case_write_files); Case.from_files of it, given the options the
    files do not carry (see case_options), rebuilds Case(cfg)."""
    lib = lib or abi.load_library()
    spec = cfg.to_spec()
    rc = lib.gfm_case_write_files(C.byref(spec), str(case_dir).encode(), runum.encode())
    if rc != abi.GFM_OK:
        raise GfmError(rc, f"gfm_case_write_files failed for {case_dir}")


def case_options(cfg: FurnaceCase) -> dict:
    """The keyword options of Case.from_files that a synthetic furnace's case
    files do not carry."""
    s = cfg.to_spec()
    return {"sigma_eps": s.sigma_eps, "wall_sink": bool(s.wall_sink), "t_wall_k": s.t_wall_k,
            "rad_emission": bool(s.rad_emission), "kappa": list(s.kappa)[:s.nwl],
            "adi_mode": s.adi_mode, "precision": s.precision}


def gflow_batch(solvers: list, n_iter: int) -> tuple[list, list]:
    """n_iter iterations of several independent solvers with their GPU work
    overlapped (gfm_gpu_gflow_batch); returns each solver's stats and count."""
    if not solvers:
        return [], []
    lib = solvers[0].lib
    n = len(solvers)
    hs = (C.c_void_p * n)(*[s.h for s in solvers])
    st = (abi.GfmIterStats * n)()
    nd = (C.c_int * n)()
    rc = lib.gfm_gpu_gflow_batch(hs, n, n_iter, st, nd)
    if rc != abi.GFM_OK:
        msgs = "; ".join(lib.gfm_gpu_last_error(s.h).decode() for s in solvers if lib.gfm_gpu_last_error(s.h))
        raise GfmError(rc, msgs)
    return [st[i].as_dict() for i in range(n)], [nd[i] for i in range(n)]


class GpuSolver:
    """GB300 SIMPLER solver for one case; fields stay resident on the device."""

    def __init__(self, case: Case, adi_mode: int | None = None, precision: int | None = None,
                 bgcon: float | None = None):
        self.case = case
        self.lib = case.lib
        n = self.lib.gfm_gpu_device_count()
        if n < 1:
            raise GfmError(n, "no CUDA device: the GB300 solver has no CPU path")
        prm = abi.GfmParams.from_buffer_copy(case.params)
        if adi_mode is not None:
            prm.adi_mode = adi_mode
        if precision is not None:
            prm.precision = precision
        if bgcon is not None:
            prm.bgcon = bgcon   # convergence threshold on res_mass (Sphase.f90:193)
        self.params = prm
        h = C.c_void_p()
        rc = self.lib.gfm_gpu_create(C.byref(case.grid), C.byref(prm), C.byref(h))
        if rc != abi.GFM_OK:
            raise GfmError(rc, self.lib.gfm_gpu_last_error(None).decode())
        self.h = h

    def _check(self, rc: int) -> None:
        if rc != abi.GFM_OK:
            raise GfmError(rc, self.lib.gfm_gpu_last_error(self.h).decode())

    def upload(self, fields: Fields) -> None:
        f = fields.to_c()
        self._check(self.lib.gfm_gpu_upload(self.h, C.byref(f)))

    def initsv(self) -> None:
        self._check(self.lib.gfm_gpu_initsv(self.h))

    def start(self) -> None:
        """Upload the case's fresh-start fields and run INITSV's interpolation."""
        self.upload(self.case.initial_fields())
        self.initsv()

    def gflow(self, n_iter: int = 1) -> tuple[dict, int]:
        st = abi.GfmIterStats()
        nd = C.c_int(0)
        self._check(self.lib.gfm_gpu_gflow(self.h, n_iter, C.byref(st), C.byref(nd)))
        return st.as_dict(), nd.value

    def download(self) -> Fields:
        out = Fields.empty(self.case.mp, self.case.np, self.case.lp)
        f = out.to_c()
        self._check(self.lib.gfm_gpu_download(self.h, C.byref(f)))
        out.update_scalars(f)
        return out

    def rad_emission(self) -> None:
        self._check(self.lib.gfm_gpu_rad_emission(self.h))

    def minor_upload(self, m: "Minor") -> None:
        """The minor species state the band model (and MSFLOW) work on."""
        self._check(self.lib.gfm_gpu_minor_upload(self.h, C.byref(m.to_c())))

    def initsvm(self, restart: bool = False) -> None:
        """INITSVM: the minor species from the major ones, or (restart) the
        uploaded state with its inlets reset and exits extrapolated."""
        self._check(self.lib.gfm_gpu_initsvm(self.h, int(restart)))

    def msflow(self, maxms: int) -> dict:
        """MSFLOW on the frozen flow; the last iteration's figures."""
        st = abi.GfmMsflowStats()
        self._check(self.lib.gfm_gpu_msflow(self.h, maxms, C.byref(st)))
        return st.as_dict()

    def minor_download(self) -> "Minor":
        out = Minor.empty(self.case.mp, self.case.np, self.case.lp)
        c = out.to_c()
        self._check(self.lib.gfm_gpu_minor_download(self.h, C.byref(c)))
        out.update_scalars(c)
        return out

    def rad_transfer(self) -> dict:
        """Volume radiation transfer from the current T (QE and QA replaced); the totals in W."""
        t = abi.GfmRadTotals()
        self._check(self.lib.gfm_gpu_rad_transfer(self.h, C.byref(t)))
        return t.as_dict()

    def wall_setup(self, spec=None) -> None:
        """Ends every later rad_transfer with the wall radiosity exchange, with
        the case's wall inputs unless `spec` is given."""
        spec = spec if spec is not None else self.case.c.wall
        self._check(self.lib.gfm_gpu_wall_setup(self.h, C.byref(spec)))

    def wall_totals(self) -> dict:
        t = abi.GfmWallTotals()
        self._check(self.lib.gfm_gpu_wall_totals(self.h, C.byref(t)))
        return t.as_dict()

    def wall_array(self, name: str) -> np.ndarray:
        out = np.zeros(self.case.grid.b_cnt)
        n = self.lib.gfm_gpu_wall_get(self.h, name.encode(), abi.dptr(out), out.size)
        if n != out.size:
            self._check(n if n < 0 else abi.GFM_E_ARG)
        return out

    def wall_vf(self) -> np.ndarray:
        """The normalised view factors, vf[n, m] from near patch n to far patch m."""
        nb = self.case.grid.b_cnt
        out = np.zeros((nb, nb))
        n = self.lib.gfm_gpu_wall_vf(self.h, abi.dptr(out), out.size)
        if n != out.size:
            self._check(n if n < 0 else abi.GFM_E_ARG)
        return out

    def wall_put(self, name: str, values) -> None:
        """Restores "radiosity" or "b_t" (per patch), or "iterw", "q_melt",
        "avg_wall_T" (one value) of the wall exchange."""
        v = np.ascontiguousarray(np.atleast_1d(values), dtype=np.float64)
        self._check(self.lib.gfm_gpu_wall_put(self.h, name.encode(), abi.dptr(v), v.size))

    def adlbl3(self, xt, ap, as6, bs, ib, ie, jb, je, kb, ke, nim) -> np.ndarray:
        x = np.ascontiguousarray(xt, dtype=np.float64).copy()
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in as6]
        ptrs = (abi._dp * 6)(*[abi.dptr(a) for a in arrs])
        self._check(self.lib.gfm_gpu_adlbl3(self.h, abi.dptr(x), abi.dptr(np.ascontiguousarray(ap, dtype=np.float64)),
                                            ptrs, abi.dptr(np.ascontiguousarray(bs, dtype=np.float64)),
                                            ib, ie, jb, je, kb, ke, nim))
        return x

    def set_lp(self, lp) -> None:
        """Start every p' solve from the network's guess (None: from zero)."""
        self._check(self.lib.gfm_gpu_set_lp(self.h, lp.h if lp is not None else None))
        self._lp = lp   # keep the network alive while the solver uses it

    def kernel_times(self) -> dict:
        a, b, c = C.c_double(), C.c_double(), C.c_double()
        n = C.c_longlong()
        self._check(self.lib.gfm_gpu_kernel_times(self.h, C.byref(a), C.byref(b), C.byref(c), C.byref(n)))
        return {"adi_ms": a.value, "gflow_ms": b.value, "other_ms": c.value, "launches": n.value}

    def iteration_profile(self) -> dict:
        k, a = C.c_longlong(), C.c_longlong()
        v = C.c_double()
        self._check(self.lib.gfm_gpu_iteration_profile(self.h, C.byref(k), C.byref(a), C.byref(v)))
        return {"kernels_per_iter": k.value, "adi_kernels_per_iter": a.value, "adi_cell_visits_per_iter": v.value}

    def reset_kernel_times(self) -> None:
        self._check(self.lib.gfm_gpu_reset_kernel_times(self.h))

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.gfm_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
