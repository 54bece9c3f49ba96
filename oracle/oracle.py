"""ctypes wrapper of the CPU oracle (oracle.cpp).  TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may use this module,
and only as the parity reference or the timed CPU baseline.  Build with ``make -C oracle`` (or
``build()`` below).  Arrays are grid SoA [species][nlev][nlat][nlon] float64.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from reseact.esm_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
_lib = None


def build(force=False):
    if force or not os.path.exists(LIB_PATH) or \
            os.path.getmtime(LIB_PATH) < os.path.getmtime(os.path.join(HERE, "oracle.cpp")):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        vp, dp = C.c_void_p, C.POINTER(C.c_double)
        L.or_create.restype = vp
        L.or_create.argtypes = [C.POINTER(abi.rs_config)]
        L.or_destroy.argtypes = [vp]
        L.or_set_lu_order.argtypes = [vp, C.POINTER(C.c_int32)]
        L.or_set_forcing.argtypes = [vp, C.POINTER(abi.rs_forcing)]
        L.or_set_rates.argtypes = [vp, dp]
        L.or_get_rates.argtypes = [vp, dp]
        L.or_cell_rates.argtypes = [vp, C.c_double, C.c_double, dp]
        L.or_rhs_transport.argtypes = [vp, C.c_double, dp, dp]
        L.or_rhs_chem.argtypes = [vp, dp, dp]
        L.or_block_jac.argtypes = [vp, dp, dp]
        L.or_single_step.restype = C.c_double
        L.or_single_step.argtypes = [vp, C.c_int, C.c_double, C.c_double, dp, dp]
        L.or_macro_step.restype = C.c_int
        L.or_macro_step.argtypes = [vp, dp, C.c_double, C.c_double, dp, dp, dp]
        L.or_chem_per_cell.restype = C.c_int
        L.or_chem_per_cell.argtypes = [vp, dp, C.c_double, C.c_double, C.c_double, dp, dp]
        L.or_reduce_fixed.restype = C.c_double
        L.or_reduce_fixed.argtypes = [dp, C.c_size_t]
        L.or_record_clear.argtypes = [vp]
        L.or_record_count.argtypes = [vp]
        L.or_record_count.restype = C.c_int
        L.or_record_macro_step.restype = C.c_int
        L.or_record_macro_step.argtypes = [vp, dp, C.c_double, C.c_double, dp, dp, dp]
        L.or_replay.argtypes = [vp, dp]
        L.or_adjoint_backward.argtypes = [vp, dp, dp]
        L.or_ssprk43_vjp.argtypes = [vp, dp, C.c_double, C.c_double, dp, dp]
        L.or_ros23_vjp.argtypes = [vp, dp, C.c_double, dp, dp, dp]
        L.or_transport_rhs_vjp.argtypes = [vp, dp, C.c_double, dp, dp]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Oracle:
    """One oracle model: mechanism + grid + forcing."""

    def __init__(self, config, forcing_abi, mech_abi=None):
        self._keep = (mech_abi, forcing_abi)
        self.cfg = config
        self.h = lib().or_create(C.byref(config))
        g = config.grid
        self.shape = (g.nlev, g.nlat, g.nlon)
        self.nc = g.nlon * g.nlat * g.nlev
        self.ns = config.mech.n_species
        self.nsp = self.ns + (1 if config.has_air_mass else 0)
        self.nr = config.mech.n_reactions
        lib().or_set_forcing(self.h, C.byref(forcing_abi.struct))

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_destroy(self.h)
            self.h = None

    def set_lu_order(self, ord=None):
        """Eliminate in this species order (as a production build does); None: natural."""
        if ord is None:
            lib().or_set_lu_order(self.h, None)
        else:
            self._ord = np.ascontiguousarray(ord, dtype=np.int32)
            lib().or_set_lu_order(self.h, self._ord.ctypes.data_as(C.POINTER(C.c_int32)))

    def set_forcing(self, forcing_abi):
        self._keep = (self._keep[0], forcing_abi)
        lib().or_set_forcing(self.h, C.byref(forcing_abi.struct))

    def rates(self):
        k = np.empty((self.nr,) + self.shape)
        lib().or_get_rates(self.h, _p(k))
        return k

    def set_rates(self, k):
        k = np.ascontiguousarray(k, dtype=np.float64)
        lib().or_set_rates(self.h, _p(k))

    def cell_rates(self, T, P):
        k = np.empty(self.nr)
        lib().or_cell_rates(self.h, T, P, _p(k))
        return k

    def rhs_transport(self, u, t=0.0):
        u = np.ascontiguousarray(u, dtype=np.float64)
        du = np.empty_like(u)
        lib().or_rhs_transport(self.h, t, _p(u), _p(du))
        return du

    def rhs_chem(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64)
        du = np.empty_like(u)
        lib().or_rhs_chem(self.h, _p(u), _p(du))
        return du

    def block_jac(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64)
        J = np.empty((self.nc, self.nsp, self.nsp))
        lib().or_block_jac(self.h, _p(u), _p(J))
        return J

    def single_step(self, op, u, t, dt):
        u = np.ascontiguousarray(u, dtype=np.float64)
        un = np.empty_like(u)
        e = lib().or_single_step(self.h, op, t, dt, _p(u), _p(un))
        return un, e

    def macro_step(self, u, t0, t1, dtT, dtC):
        """In place on u (grid SoA).  Returns (status, dtT, dtC, stats[8])."""
        assert u.flags.c_contiguous and u.dtype == np.float64
        a, b = C.c_double(dtT), C.c_double(dtC)
        st = np.zeros(8)
        rc = lib().or_macro_step(self.h, _p(u), t0, t1, C.byref(a), C.byref(b), _p(st))
        return rc, a.value, b.value, st

    def chem_per_cell(self, u, t0, t1, dt0, dt_cell=None):
        """Per-cell adaptive chemistry over [t0, t1], in place on u (grid SoA).  dt_cell (may be
        None): per-cell step sizes carried in (<= 0: start from dt0); returns (status, the
        carried step sizes, accepted steps per cell)."""
        assert u.flags.c_contiguous and u.dtype == np.float64
        dt = np.zeros(self.nc) if dt_cell is None else np.array(dt_cell, dtype=np.float64)
        steps = np.empty(self.nc)
        rc = lib().or_chem_per_cell(self.h, _p(u), t0, t1, dt0, _p(dt), _p(steps))
        return rc, dt, steps

    # ---------------------------------------------------------------- discrete adjoint
    def record_clear(self):
        lib().or_record_clear(self.h)

    def record_macro_step(self, u, t0, t1, dtT, dtC):
        assert u.flags.c_contiguous and u.dtype == np.float64
        a, b = C.c_double(dtT), C.c_double(dtC)
        st = np.zeros(8)
        rc = lib().or_record_macro_step(self.h, _p(u), t0, t1, C.byref(a), C.byref(b), _p(st))
        return rc, a.value, b.value, st

    def replay(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64).copy()
        lib().or_replay(self.h, _p(u))
        return u

    def adjoint_backward(self, lam_end):
        lam = np.ascontiguousarray(lam_end, dtype=np.float64).copy()
        ebar = np.zeros((self.ns,) + self.shape)
        lib().or_adjoint_backward(self.h, _p(lam), _p(ebar))
        return lam, ebar

    def ssprk43_vjp(self, u, t, dt, lam):
        u = np.ascontiguousarray(u, dtype=np.float64)
        lam = np.ascontiguousarray(lam, dtype=np.float64)
        out = np.empty_like(u)
        lib().or_ssprk43_vjp(self.h, _p(u), t, dt, _p(lam), _p(out))
        return out

    def ros23_vjp(self, u, dt, lam):
        u = np.ascontiguousarray(u, dtype=np.float64)
        lam = np.ascontiguousarray(lam, dtype=np.float64)
        out = np.empty_like(u)
        ebar = np.zeros((self.ns,) + self.shape)
        lib().or_ros23_vjp(self.h, _p(u), dt, _p(lam), _p(out), _p(ebar))
        return out, ebar

    def transport_rhs_vjp(self, u, t, fbar):
        u = np.ascontiguousarray(u, dtype=np.float64)
        fbar = np.ascontiguousarray(fbar, dtype=np.float64)
        out = np.empty_like(u)
        lib().or_transport_rhs_vjp(self.h, _p(u), t, _p(fbar), _p(out))
        return out


def reduce_fixed(e):
    e = np.ascontiguousarray(e, dtype=np.float64)
    return lib().or_reduce_fixed(_p(e), e.size)


def box_model(mech, tol=1e-9, atol=1e-16):
    """A one-cell chemistry-only oracle (the 0-D box model of the .esm golden tests)."""
    from reseact.esm_gb300 import workloads
    g = workloads.latlon_grid(1, 1, 1, pole_centred=False)
    mabi = abi.MechanismABI(mech)
    cfg = abi.make_config(g, mabi, has_air_mass=False, do_transport=False, rtol=tol,
                          atol_C=atol, maxiters=1e6, clamp_nonneg=False)
    return mabi, cfg
