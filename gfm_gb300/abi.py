"""ctypes mirror of include/gfm_gb300.h and loader for the native library.

The structures below must match the C header field for field; the test
``tests/test_abi.py`` checks the library exports every declared symbol.
"""
from __future__ import annotations

import ctypes as C
import os
import pathlib

import numpy as np

PKG_DIR = pathlib.Path(__file__).resolve().parent
LIB_PATH = PKG_DIR / "libgfm_gb300.so"
KINETIC_PATH = PKG_DIR / "data" / "kinetic.d"

GFM_OK = 0
GFM_E_ARG = -1
GFM_E_CUDA = -2
GFM_E_NAN = -3
GFM_E_UNSUPPORTED = -4
GFM_E_NOMEM = -5
GFM_E_TIMEOUT = -6
GFM_E_NODEVICE = -7
GFM_E_LIMIT = -8
GFM_E_IO = -9

GFM_ADI_MARCH = 0
GFM_ADI_REDBLACK = 1
GFM_PREC_FP64 = 0
GFM_PREC_MIXED = 1

_dp = C.POINTER(C.c_double)
_i16p = C.POINTER(C.c_int16)


class GfmGrid(C.Structure):
    _fields_ = [
        ("mp", C.c_int), ("np", C.c_int), ("lp", C.c_int),
        ("x", _dp), ("dx", _dp), ("r", _dp), ("dr", _dp), ("rs", _dp), ("z", _dp), ("dz", _dp),
        ("ibcell", _i16p),
        ("ncells", C.c_int),
        ("i_ref", C.c_int), ("j_ref", C.c_int), ("k_ref", C.c_int),
        ("p_ref", C.c_double),
        ("b_cnt", C.c_int),
        ("b_typ", _i16p), ("b_i", _i16p), ("b_j", _i16p), ("b_k", _i16p),
        ("b_orient", _i16p), ("b_direct", _i16p),
        ("b_t", _dp),
        ("nr0", C.c_int),
        ("rtim", _dp), ("delrt", _dp), ("hrt", _dp), ("delr", _dp), ("timed", _dp), ("hrd", _dp),
        ("nwl", C.c_int),
        ("wl", _dp), ("akl0", _dp),
        ("bv_f", C.c_double * 2), ("ba_f", C.c_double * 6),
    ]


class GfmParams(C.Structure):
    _fields_ = [
        ("t0", C.c_double), ("h_0", C.c_double), ("dnst0", C.c_double), ("ug0", C.c_double),
        ("gmfr", C.c_double), ("pg0", C.c_double), ("r0", C.c_double),
        ("reyg", C.c_double), ("reyg2", C.c_double), ("epsr", C.c_double), ("taur", C.c_double),
        ("eun", C.c_double), ("qr0", C.c_double), ("q0", C.c_double), ("tk0", C.c_double),
        ("gra", C.c_double * 3),
        ("amu", C.c_double), ("trdg", C.c_double), ("wt0", C.c_double), ("stoich", C.c_double),
        ("cmu", C.c_double), ("ct1", C.c_double), ("ct2", C.c_double),
        ("p_mx", C.c_double), ("p_mn", C.c_double), ("t_mx", C.c_double), ("t_mn", C.c_double),
        ("u_mx", C.c_double), ("u_mn", C.c_double), ("f_mx", C.c_double), ("f_mn", C.c_double),
        ("rf", C.c_double * 21), ("rfl", C.c_double * 21),
        ("sigma", C.c_double * 12),
        ("ntimesg", C.c_int * 20),
        ("rf_hsource", C.c_double),
        ("react", C.c_int), ("turb", C.c_int),
        ("wall_sink", C.c_int), ("h_g", C.c_double),
        ("rad_emission", C.c_int), ("rad_qe_frequency", C.c_int),
        ("sig", C.c_double), ("ri", C.c_double), ("hck", C.c_double),
        ("bgcon", C.c_double),
        ("maxgi", C.c_int),
        ("adi_mode", C.c_int),
        ("precision", C.c_int),
        ("gas_model", C.c_int), ("maxms", C.c_int), ("ntimesm", C.c_int), ("irstypm", C.c_int),
        ("bmcon", C.c_double), ("ssigma", C.c_double), ("rfm", C.c_double), ("rfm_soot", C.c_double),
        ("rf_soot_form", C.c_double), ("rf_soot_oxid", C.c_double),
        ("soot_cap", C.c_double), ("t0_sf", C.c_double), ("t0_so", C.c_double),
        ("aform", C.c_double), ("aoxid", C.c_double), ("esf_r", C.c_double), ("eso_r", C.c_double),
    ]


class GfmFields(C.Structure):
    _fields_ = [
        ("p", _dp), ("t", _dp), ("dnst", _dp), ("theta", _dp), ("tmu", _dp), ("gama", _dp),
        ("crate", _dp), ("hrate", _dp), ("bs_hprev", _dp),
        ("ug", _dp), ("gf", _dp), ("qa", _dp), ("qe", _dp),
        ("itr_gas", C.c_int), ("do_rad_qe_only_cnt", C.c_int), ("i1st_rad_qe_done", C.c_int),
        ("factor", C.c_double), ("fadj", C.c_double), ("gfin0", C.c_double), ("q_h_in", C.c_double),
    ]


NSP_MINOR = 7


class GfmMinor(C.Structure):
    _fields_ = [
        ("gfm", _dp), ("smf", _dp), ("bs_soot_prev", _dp), ("sfp_soot_prev", _dp), ("rrms", _dp),
        ("itr_ms", C.c_int), ("imscon", C.c_int),
    ]


class GfmMsflowStats(C.Structure):
    _fields_ = [
        ("itr_ms", C.c_int), ("iterations", C.c_int), ("converged", C.c_int), ("reserved", C.c_int),
        ("resid_ms_pre", C.c_double * 8), ("resid_ms", C.c_double * 8),
        ("bal_ms", C.c_double), ("soot_tot", C.c_double), ("smf_max", C.c_double), ("smf_max_noclip", C.c_double),
        ("gfm_out", C.c_double * 7), ("svf_r", C.c_double),
    ]

    def as_dict(self) -> dict:
        return {"itr_ms": self.itr_ms, "iterations": self.iterations, "converged": self.converged,
                "resid_ms_pre": list(self.resid_ms_pre), "resid_ms": list(self.resid_ms), "bal_ms": self.bal_ms,
                "soot_tot": self.soot_tot, "smf_max": self.smf_max, "smf_max_noclip": self.smf_max_noclip,
                "gfm_out": list(self.gfm_out), "svf_r": self.svf_r}


class GfmIterStats(C.Structure):
    _fields_ = [
        ("itr_gas", C.c_int), ("converged", C.c_int),
        ("res_mass", C.c_double), ("res_mass_max", C.c_double),
        ("p_resid_pre", C.c_double), ("p_resid", C.c_double), ("pcorr_resid", C.c_double),
        ("u_resid_pre", C.c_double * 3), ("u_resid", C.c_double * 3),
        ("gf_resid_pre", C.c_double * 10), ("gf_resid", C.c_double * 10),
        ("factor", C.c_double), ("gfin", C.c_double), ("gfex", C.c_double),
        ("q_react", C.c_double), ("q_exhaust", C.c_double), ("q_conv_total", C.c_double),
        ("q_global_bal", C.c_double),
        ("tave", C.c_double), ("tmean_ex", C.c_double),
        ("lp_used", C.c_int), ("lp_ratio", C.c_double),
    ]

    def as_dict(self) -> dict:
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            out[name] = list(v) if isinstance(v, C.Array) else v
        return out


class GfmRadTotals(C.Structure):
    _fields_ = [
        ("qe_sum_from_open", C.c_double), ("qa_sum_to_open", C.c_double),
        ("qa_sum_to_wall", C.c_double), ("qa_sum_to_inlet", C.c_double), ("qa_sum_to_exit", C.c_double),
        ("qa_sum_to_melt", C.c_double),
        ("tot_qe_h2o_co2", C.c_double), ("tot_qe_soot", C.c_double),
        ("n_emitters", C.c_int), ("reserved", C.c_int),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_ if name != "reserved"}


class GfmInletSpec(C.Structure):
    _fields_ = [
        ("y0", C.c_double), ("y1", C.c_double), ("z0", C.c_double), ("z1", C.c_double),
        ("t_k", C.c_double),
        ("yf", C.c_double), ("yo2", C.c_double), ("yn2", C.c_double), ("yco2", C.c_double), ("yh2o", C.c_double),
        ("u_ms", C.c_double),
    ]


class GfmCaseSpec(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("lx", C.c_double), ("ly", C.c_double), ("lz", C.c_double),
        ("n_inlets", C.c_int),
        ("inlets", GfmInletSpec * 8),
        ("exit_y0", C.c_double), ("exit_y1", C.c_double), ("exit_z0", C.c_double), ("exit_z1", C.c_double),
        ("t_init_k", C.c_double), ("noise_amp", C.c_double),
        ("seed", C.c_uint64),
        ("inlet_jitter", C.c_double),
        ("t_wall_k", C.c_double),
        ("rf_uvw", C.c_double), ("rfl_h", C.c_double), ("rfl_k", C.c_double), ("rfl_eps", C.c_double),
        ("rfl_species", C.c_double), ("rf_hsource", C.c_double),
        ("ntimesg", C.c_int * 12),
        ("sigma_k", C.c_double), ("sigma_eps", C.c_double),
        ("nwl", C.c_int),
        ("kappa", C.c_double * 16), ("wl_um", C.c_double * 16),
        ("pg0", C.c_double), ("q0_jkg", C.c_double), ("h_g", C.c_double),
        ("react", C.c_int), ("wall_sink", C.c_int), ("rad_emission", C.c_int), ("maxgi", C.c_int),
        ("bgcon", C.c_double),
        ("adi_mode", C.c_int), ("precision", C.c_int),
    ]


class GfmRestartTail(C.Structure):
    _fields_ = [
        ("mz", C.c_int), ("nz", C.c_int), ("t_surf_prev", _dp),
        ("i1st_rad_done", C.c_int), ("itr_rad", C.c_int), ("itr_gend", C.c_int), ("interval_rad", C.c_int),
    ]


MAX_EXHAUSTS = 16


class GfmWallSpec(C.Structure):
    _fields_ = [
        ("eps_w", C.c_double), ("eps_c", C.c_double), ("eps_m", C.c_double),
        ("have_crown", C.c_int), ("height_to_ceiling", C.c_double),
        ("maxri1", C.c_int), ("maxri2", C.c_int), ("minri2", C.c_int),
        ("t_a", C.c_double), ("h_a", C.c_double), ("w_k", C.c_double), ("w_d", C.c_double),
        ("t_mnk", C.c_double),
        ("nex", C.c_int),
    ] + [(n, C.c_int * MAX_EXHAUSTS) for n in ("exh_i1", "exh_j1", "exh_k1", "exh_i2", "exh_j2", "exh_k2",
                                                "exh_orient", "exh_direct", "exh_type")] + [
        ("exh_frac", C.c_double * MAX_EXHAUSTS), ("exh_fixed", C.c_double * MAX_EXHAUSTS),
    ]


class GfmWallTotals(C.Structure):
    _fields_ = [("b_cnt", C.c_int), ("sweeps", C.c_int), ("outer", C.c_int), ("reserved", C.c_int)] + [
        (n, C.c_double) for n in ("avg_wall_T", "q_melt", "q_wall_loss", "q_incident_total", "q_incident_wall",
                                  "q_incident_inlet", "q_incident_exit", "q_incident_melt", "qconv_total",
                                  "q_rad_inlet", "q_rad_outlet", "qm_flame", "qm_bnds", "qm_conv",
                                  "rel_rad_chg_mean")]

    def as_dict(self) -> dict:
        return {n: getattr(self, n) for n, _ in self._fields_ if n != "reserved"}


class GfmCase(C.Structure):
    _fields_ = [("grid", GfmGrid), ("params", GfmParams), ("fields", GfmFields), ("priv", C.c_void_p),
                ("tail", GfmRestartTail), ("wall", GfmWallSpec)]


class GfmCaseFiles(C.Structure):
    _fields_ = [("gd", C.c_char_p), ("sbc", C.c_char_p), ("relax", C.c_char_p), ("it", C.c_char_p),
                ("rg", C.c_char_p), ("kinetic", C.c_char_p), ("rr", C.c_char_p)]


class GfmCaseOptions(C.Structure):
    _fields_ = [
        ("sigma_eps", C.c_double), ("wall_sink", C.c_int), ("t_wall_k", C.c_double), ("rad_emission", C.c_int),
        ("kappa", C.c_double * 16), ("maxgi", C.c_int), ("adi_mode", C.c_int), ("precision", C.c_int),
        ("gas_model", C.c_int),
    ]


class GfmCaseSummary(C.Structure):
    _fields_ = [
        ("ncells", C.c_int), ("area_melt_surf", C.c_double),
        ("fr_f", C.c_double), ("fr_ox", C.c_double), ("fr_n2", C.c_double),
        ("heat_in_fuel", C.c_double), ("q_h_in", C.c_double), ("gmfr", C.c_double), ("gfin0", C.c_double),
        ("irstyp", C.c_int), ("id_rad", C.c_int), ("interval_rad", C.c_int),
        ("n_inlet_blocks", C.c_int), ("n_exhausts", C.c_int), ("n_wall_blocks", C.c_int), ("n_melt_cells", C.c_int),
        ("restarted", C.c_int), ("itr_gas", C.c_int),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


# (name, restype, argtypes) of every entry point declared in include/gfm_gb300.h
SIGNATURES = [
    ("gfm_case_build", C.c_int, [C.POINTER(GfmCaseSpec), C.c_char_p, C.POINTER(GfmCase)]),
    ("gfm_case_free", None, [C.POINTER(GfmCase)]),
    ("gfm_case_read", C.c_int, [C.POINTER(GfmCaseFiles), C.POINTER(GfmCaseOptions), C.POINTER(GfmCase),
                                C.POINTER(GfmCaseSummary)]),
    ("gfm_restart_write", C.c_int, [C.c_char_p, C.POINTER(GfmGrid), C.POINTER(GfmFields), C.POINTER(GfmRestartTail)]),
    ("gfm_case_write_files", C.c_int, [C.POINTER(GfmCaseSpec), C.c_char_p, C.c_char_p]),
    ("gfm_gpu_device_count", C.c_int, []),
    ("gfm_gpu_create", C.c_int, [C.POINTER(GfmGrid), C.POINTER(GfmParams), C.POINTER(C.c_void_p)]),
    ("gfm_gpu_upload", C.c_int, [C.c_void_p, C.POINTER(GfmFields)]),
    ("gfm_gpu_initsv", C.c_int, [C.c_void_p]),
    ("gfm_gpu_gflow", C.c_int, [C.c_void_p, C.c_int, C.POINTER(GfmIterStats), C.POINTER(C.c_int)]),
    ("gfm_gpu_gflow_batch", C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.c_int, C.POINTER(GfmIterStats),
                                      C.POINTER(C.c_int)]),
    ("gfm_gpu_download", C.c_int, [C.c_void_p, C.POINTER(GfmFields)]),
    ("gfm_gpu_adlbl3", C.c_int, [C.c_void_p, _dp, _dp, C.POINTER(_dp), _dp,
                                 C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]),
    ("gfm_gpu_rad_emission", C.c_int, [C.c_void_p]),
    ("gfm_gpu_rad_transfer", C.c_int, [C.c_void_p, C.POINTER(GfmRadTotals)]),
    ("gfm_gpu_wall_setup", C.c_int, [C.c_void_p, C.POINTER(GfmWallSpec)]),
    ("gfm_gpu_wall_totals", C.c_int, [C.c_void_p, C.POINTER(GfmWallTotals)]),
    ("gfm_gpu_wall_get", C.c_int, [C.c_void_p, C.c_char_p, _dp, C.c_int]),
    ("gfm_gpu_wall_vf", C.c_longlong, [C.c_void_p, _dp, C.c_longlong]),
    ("gfm_gpu_wall_put", C.c_int, [C.c_void_p, C.c_char_p, _dp, C.c_int]),
    ("gfm_minor_read", C.c_int, [C.c_char_p, C.POINTER(GfmGrid), C.POINTER(GfmMinor)]),
    ("gfm_minor_write", C.c_int, [C.c_char_p, C.POINTER(GfmGrid), C.POINTER(GfmMinor)]),
    ("gfm_gpu_minor_upload", C.c_int, [C.c_void_p, C.POINTER(GfmMinor)]),
    ("gfm_gpu_minor_download", C.c_int, [C.c_void_p, C.POINTER(GfmMinor)]),
    ("gfm_gpu_initsvm", C.c_int, [C.c_void_p, C.c_int]),
    ("gfm_gpu_msflow", C.c_int, [C.c_void_p, C.c_int, C.POINTER(GfmMsflowStats)]),
    ("gfm_gpu_kernel_times", C.c_int, [C.c_void_p, _dp, _dp, _dp, C.POINTER(C.c_longlong)]),
    ("gfm_gpu_reset_kernel_times", C.c_int, [C.c_void_p]),
    ("gfm_gpu_iteration_profile", C.c_int, [C.c_void_p, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong), _dp]),
    ("gfm_gpu_last_error", C.c_char_p, [C.c_void_p]),
    ("gfm_gpu_destroy", None, [C.c_void_p]),
    ("gfm_lp_create", C.c_int, [C.c_int, C.c_int, C.c_int, C.c_uint64, C.POINTER(C.c_void_p)]),
    ("gfm_lp_destroy", None, [C.c_void_p]),
    ("gfm_lp_num_params", C.c_int, []),
    ("gfm_lp_get_params", C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    ("gfm_lp_set_params", C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
    ("gfm_lp_forward", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p]),
    ("gfm_lp_train_step", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_float,
                                    C.c_int, C.POINTER(C.c_double), C.c_void_p]),
    ("gfm_lp_set_tensor_path", C.c_int, [C.c_void_p, C.c_int]),
    ("gfm_lp_tensor_status", C.c_int, [C.c_void_p]),
    ("gfm_lp_last_error", C.c_char_p, []),
    ("gfm_gpu_pcorr_sample", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.POINTER(C.c_int)]),
    ("gfm_gpu_set_lp", C.c_int, [C.c_void_p, C.c_void_p]),
    ("gfm_adlbl3_noalloc", C.c_int, [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.POINTER(C.c_void_p), C.c_void_p] + [C.c_int] * 7 + [C.c_void_p]),
]

_lib = None


class NativeLibraryMissing(RuntimeError):
    """The compiled library is absent: there is no fallback path."""


def load_library(path: os.PathLike | str | None = None) -> C.CDLL:
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = pathlib.Path(path) if path is not None else LIB_PATH
    if not p.exists():
        raise NativeLibraryMissing(
            f"{p} not found: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(str(p))
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)
