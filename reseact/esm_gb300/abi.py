"""ctypes mirror of include/reseact_gb300.h (structs, enums, defaults).

Kept in one place so the library binding (``_lib.py``) and any other C-ABI caller build the
exact same structs.  The defaults are the reference's: tolerances ``run_reseact.jl:158`` /
``run_reseact_reactant.jl:144`` (rtol 1e-4, atol 1e-6 transport, 1e-9 chemistry) and the
PI-controller constants ``tools/reactant_handoff/rx_traced_integrator.jl:86-99``.
"""
import ctypes as C

import numpy as np

RS_API_VERSION = 1
RS_OK, RS_ERR_INVALID, RS_ERR_CUDA, RS_ERR_MAXITERS, RS_ERR_NONFINITE = 0, 1, 2, 3, 4
RS_ERR_NOMEM, RS_ERR_STATE, RS_ERR_UNSUPPORTED = 5, 6, 7
STATUS_NAMES = {0: "OK", 1: "INVALID", 2: "CUDA", 3: "MAXITERS", 4: "NONFINITE", 5: "NOMEM",
                6: "STATE", 7: "UNSUPPORTED"}
RS_BC_PERIODIC, RS_BC_OPEN, RS_BC_CLOSED = 0, 1, 2
RS_PREC_FP64, RS_PREC_MIXED = 0, 1
RS_CHEM_GLOBAL_DT, RS_CHEM_PER_CELL = 0, 1
RS_OP_TRANSPORT, RS_OP_CHEMISTRY = 0, 1

_i32p = C.POINTER(C.c_int32)
_f64p = C.POINTER(C.c_double)


class rs_mechanism(C.Structure):
    _fields_ = [("n_species", C.c_int32), ("n_reactions", C.c_int32), ("n_params", C.c_int32),
                ("combinatoric", C.c_int32),
                ("react_ptr", _i32p), ("react_species", _i32p), ("react_nu", _i32p),
                ("prod_ptr", _i32p), ("prod_species", _i32p), ("prod_coef", _f64p),
                ("prog_ptr", _i32p), ("prog_op", _i32p), ("prog_val", _f64p),
                ("params", _f64p)]


class rs_grid(C.Structure):
    _fields_ = [("nlon", C.c_int32), ("nlat", C.c_int32), ("nlev", C.c_int32),
                ("lon_bc", C.c_int32), ("lat_bc", C.c_int32),
                ("lon0_deg", C.c_double), ("dlon_deg", C.c_double),
                ("lat0_deg", C.c_double), ("dlat_deg", C.c_double)]


class rs_controller(C.Structure):
    _fields_ = [(n, C.c_double) for n in
                ("beta1", "beta2", "qmin", "qmax", "gamma", "qsteady_min", "qsteady_max",
                 "qoldinit")]


class rs_config(C.Structure):
    _fields_ = [("api_version", C.c_int32), ("device", C.c_int32), ("grid", rs_grid),
                ("has_air_mass", C.c_int32), ("do_transport", C.c_int32),
                ("do_chemistry", C.c_int32), ("mech", rs_mechanism),
                ("rtol_T", C.c_double), ("atol_T", C.c_double),
                ("rtol_C", C.c_double), ("atol_C", C.c_double),
                ("ctrl_T", rs_controller), ("ctrl_C", rs_controller),
                ("maxiters", C.c_double), ("clamp_nonneg", C.c_int32),
                ("precision", C.c_int32), ("chem_mode", C.c_int32)]


class rs_forcing(C.Structure):
    _fields_ = [("mx", _f64p), ("my", _f64p), ("mz", _f64p), ("flux_omega", C.c_double),
                ("dp", _f64p), ("qbc_w", _f64p), ("qbc_e", _f64p), ("qbc_s", _f64p),
                ("qbc_n", _f64p), ("temperature", _f64p), ("pressure", _f64p),
                ("emission", _f64p), ("pblh", _f64p), ("ps", _f64p), ("hyb_a", _f64p),
                ("hyb_b", _f64p), ("tau_pblmix", C.c_double), ("dps_dt", _f64p)]


class rs_stats(C.Structure):
    _fields_ = [("naT", C.c_double), ("nrT", C.c_double), ("naC", C.c_double),
                ("nrC", C.c_double), ("dtT_end", C.c_double), ("dtC_end", C.c_double),
                ("tT_end", C.c_double), ("tC_end", C.c_double),
                ("chem_cell_steps", C.c_double), ("kernel_launches", C.c_double),
                ("status", C.c_int32)]


REFRESH_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_double)
BISECT_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_double, C.c_double)


class rs_solve_opts(C.Structure):
    _fields_ = [("macro_dt", C.c_double), ("min_macro_dt", C.c_double),
                ("forcing_tstops", _f64p), ("n_tstops", C.c_size_t),
                ("refresh", REFRESH_FN), ("on_bisect", BISECT_FN), ("user", C.c_void_p)]


class rs_solve_result(C.Structure):
    _fields_ = [("naT", C.c_double), ("nrT", C.c_double), ("naC", C.c_double),
                ("nrC", C.c_double), ("nmacro", C.c_double), ("nbisect", C.c_double),
                ("nrefresh", C.c_double), ("status", C.c_int32), ("pad", C.c_int32)]


def pictrl_ros23():
    return rs_controller(7 / 20, 1 / 5, 1 / 5, 10.0, 9 / 10, 1.0, 6 / 5, 1e-4)


def pictrl_ssprk43():
    return rs_controller(7 / 30, 2 / 15, 1 / 5, 10.0, 9 / 10, 1.0, 1.0, 1e-4)


def _ptr(a, ctype):
    if a is None:
        return C.cast(None, C.POINTER(ctype))
    return a.ctypes.data_as(C.POINTER(ctype))


class MechanismABI:
    """Keeps the numpy tables alive while an rs_mechanism points into them."""

    def __init__(self, mech):
        t = mech.tables()
        prod_ptr, prod_sp, prod_c = [0], [], []
        for rx in mech.reactions:
            for s, c in rx.products:
                prod_sp.append(s)
                prod_c.append(c)
            prod_ptr.append(len(prod_sp))
        self.arrays = dict(
            react_ptr=t["react_ptr"], react_species=t["react_species"], react_nu=t["react_nu"],
            prod_ptr=np.asarray(prod_ptr, np.int32), prod_species=np.asarray(prod_sp, np.int32),
            prod_coef=np.asarray(prod_c, np.float64),
            prog_ptr=t["prog_ptr"], prog_op=t["prog_op"], prog_val=t["prog_val"],
            params=np.asarray(t["params"] if len(t["params"]) else np.zeros(1), np.float64))
        a = self.arrays
        self.struct = rs_mechanism(
            mech.ns, mech.nr, len(mech.params), int(mech.combinatoric),
            _ptr(a["react_ptr"], C.c_int32), _ptr(a["react_species"], C.c_int32),
            _ptr(a["react_nu"], C.c_int32), _ptr(a["prod_ptr"], C.c_int32),
            _ptr(a["prod_species"], C.c_int32), _ptr(a["prod_coef"], C.c_double),
            _ptr(a["prog_ptr"], C.c_int32), _ptr(a["prog_op"], C.c_int32),
            _ptr(a["prog_val"], C.c_double), _ptr(a["params"], C.c_double))


def make_config(grid, mech_abi, has_air_mass=True, do_transport=True, do_chemistry=True,
                precision=RS_PREC_FP64, chem_mode=RS_CHEM_GLOBAL_DT, rtol=1e-4, atol_T=1e-6,
                atol_C=1e-9, maxiters=2.0e4, clamp_nonneg=True, device=0):
    g = rs_grid(grid["nlon"], grid["nlat"], grid["nlev"], grid.get("lon_bc", RS_BC_PERIODIC),
                grid.get("lat_bc", RS_BC_CLOSED), grid.get("lon0_deg", 0.0),
                grid.get("dlon_deg", 360.0 / grid["nlon"]), grid.get("lat0_deg", 0.0),
                grid.get("dlat_deg", 1.0))
    return rs_config(RS_API_VERSION, device, g, int(has_air_mass), int(do_transport),
                     int(do_chemistry), mech_abi.struct, rtol, atol_T, rtol, atol_C,
                     pictrl_ssprk43(), pictrl_ros23(), maxiters, int(clamp_nonneg),
                     precision, chem_mode)


class ForcingABI:
    """Keeps forcing arrays alive (contiguous float64) behind an rs_forcing struct."""

    NAMES = ("mx", "my", "mz", "dp", "qbc_w", "qbc_e", "qbc_s", "qbc_n", "temperature",
             "pressure", "emission", "pblh", "ps", "hyb_a", "hyb_b", "dps_dt")

    def __init__(self, flux_omega=0.0, tau_pblmix=0.0, **arrays):
        self.arrays = {k: (None if arrays.get(k) is None else
                           np.ascontiguousarray(arrays[k], dtype=np.float64))
                       for k in self.NAMES}
        a = self.arrays
        self.struct = rs_forcing(_ptr(a["mx"], C.c_double), _ptr(a["my"], C.c_double),
                                 _ptr(a["mz"], C.c_double), float(flux_omega),
                                 _ptr(a["dp"], C.c_double), _ptr(a["qbc_w"], C.c_double),
                                 _ptr(a["qbc_e"], C.c_double), _ptr(a["qbc_s"], C.c_double),
                                 _ptr(a["qbc_n"], C.c_double),
                                 _ptr(a["temperature"], C.c_double),
                                 _ptr(a["pressure"], C.c_double),
                                 _ptr(a["emission"], C.c_double),
                                 _ptr(a["pblh"], C.c_double), _ptr(a["ps"], C.c_double),
                                 _ptr(a["hyb_a"], C.c_double), _ptr(a["hyb_b"], C.c_double),
                                 float(tau_pblmix), _ptr(a["dps_dt"], C.c_double))
