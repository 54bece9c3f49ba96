"""ctypes binding of libreseact_gb300.so -- the same C ABI a Julia ``ccall`` binds.

There is no fallback: if the CUDA library is missing or cannot load, ``load()`` raises.
"""
import ctypes as C
import os

import numpy as np

from . import abi, build

_LIBS = {}

SYMBOLS = [
    "rs_default_config", "rs_create", "rs_destroy", "rs_last_error", "rs_state_size",
    "rs_species_per_cell", "rs_set_state", "rs_get_state", "rs_set_forcing",
    "rs_get_rate_constants", "rs_set_rate_constants", "rs_get_cell_steps", "rs_macro_step",
    "rs_rhs_transport",
    "rs_rhs_chem", "rs_block_jac", "rs_single_step", "rs_state_device_ptr", "rs_stream",
    "rs_set_profiling", "rs_get_profile", "rs_reset_profile", "rs_ros23_attempt_noalloc",
    "rs_record", "rs_record_count", "rs_set_adjoint_tape", "rs_record_taped",
    "rs_adjoint_set_lambda", "rs_adjoint_get_lambda",
    "rs_backward_macro_step", "rs_adjoint_get_grad_emission", "rs_adjoint_reset_grad",
    "rs_replay_macro_step",
    "rs_autotune", "rs_set_chem_kernel", "rs_get_chem_kernel", "rs_chem_kernel_source",
    "rs_chem_kernel_compile", "rs_chem_kernel_reciprocal", "rs_lu_order",
    "rs_mechanism_lu_order", "rs_continuity_drift", "rs_lie_trotter_solve",
    "rs_set_transport_staging", "rs_get_transport_staging", "rs_set_launch_shape",
]

CHEM_KERNEL_AUTO, CHEM_KERNEL_TABLE, CHEM_KERNEL_SPECIALIZED = 0, 1, 2
STAGING_AUTO, STAGING_PLAIN, STAGING_BULK = 0, 1, 2


class RsError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s (%s)" % (msg, abi.STATUS_NAMES.get(status, status)))
        self.status = status


def _declare(L):
    vp, dp, sz = C.c_void_p, C.POINTER(C.c_double), C.c_size_t
    i32 = C.c_int32
    L.rs_default_config.argtypes = [C.POINTER(abi.rs_config)]
    L.rs_create.argtypes = [C.POINTER(abi.rs_config), C.POINTER(vp)]
    L.rs_create.restype = C.c_int
    L.rs_destroy.argtypes = [vp]
    L.rs_last_error.argtypes = [vp]
    L.rs_last_error.restype = C.c_char_p
    L.rs_state_size.argtypes = [vp]
    L.rs_state_size.restype = sz
    L.rs_species_per_cell.argtypes = [vp]
    L.rs_species_per_cell.restype = i32
    for f in ("rs_set_state", "rs_get_state"):
        getattr(L, f).argtypes = [vp, dp, sz]
        getattr(L, f).restype = C.c_int
    L.rs_set_forcing.argtypes = [vp, C.POINTER(abi.rs_forcing)]
    L.rs_set_forcing.restype = C.c_int
    for f in ("rs_get_rate_constants", "rs_set_rate_constants"):
        getattr(L, f).argtypes = [vp, dp, sz]
        getattr(L, f).restype = C.c_int
    L.rs_get_cell_steps.argtypes = [vp, dp, dp, sz]
    L.rs_get_cell_steps.restype = C.c_int
    L.rs_macro_step.argtypes = [vp, C.c_double, C.c_double, dp, dp, C.POINTER(abi.rs_stats)]
    L.rs_macro_step.restype = C.c_int
    for f in ("rs_rhs_transport", "rs_rhs_chem"):
        getattr(L, f).argtypes = [vp, C.c_double, dp, dp, sz]
        getattr(L, f).restype = C.c_int
    L.rs_block_jac.argtypes = [vp, dp, dp, sz]
    L.rs_block_jac.restype = C.c_int
    L.rs_single_step.argtypes = [vp, i32, C.c_double, C.c_double, dp, dp, dp, sz]
    L.rs_single_step.restype = C.c_int
    L.rs_state_device_ptr.argtypes = [vp, C.POINTER(vp)]
    L.rs_state_device_ptr.restype = C.c_int
    L.rs_stream.argtypes = [vp]
    L.rs_stream.restype = vp
    L.rs_set_profiling.argtypes = [vp, i32]
    L.rs_set_profiling.restype = C.c_int
    L.rs_reset_profile.argtypes = [vp]
    L.rs_reset_profile.restype = C.c_int
    L.rs_get_profile.argtypes = [vp, C.c_char_p, sz, dp, dp, i32, C.POINTER(i32)]
    L.rs_get_profile.restype = C.c_int
    L.rs_ros23_attempt_noalloc.argtypes = [vp, C.c_double, vp, vp, dp]
    L.rs_ros23_attempt_noalloc.restype = C.c_int
    L.rs_record.argtypes = [vp, i32]
    L.rs_record.restype = C.c_int
    L.rs_record_count.argtypes = [vp]
    L.rs_record_count.restype = i32
    L.rs_set_adjoint_tape.argtypes = [vp, C.c_int64]
    L.rs_set_adjoint_tape.restype = C.c_int
    L.rs_record_taped.argtypes = [vp]
    L.rs_record_taped.restype = i32
    for f in ("rs_adjoint_set_lambda", "rs_adjoint_get_lambda", "rs_adjoint_get_grad_emission"):
        getattr(L, f).argtypes = [vp, dp, sz]
        getattr(L, f).restype = C.c_int
    L.rs_backward_macro_step.argtypes = [vp, i32]
    L.rs_backward_macro_step.restype = C.c_int
    L.rs_replay_macro_step.argtypes = [vp, i32]
    L.rs_replay_macro_step.restype = C.c_int
    L.rs_adjoint_reset_grad.argtypes = [vp]
    L.rs_adjoint_reset_grad.restype = C.c_int
    L.rs_autotune.argtypes = [vp, C.c_char_p, sz]
    L.rs_autotune.restype = C.c_int
    L.rs_set_chem_kernel.argtypes = [vp, i32]
    L.rs_set_chem_kernel.restype = C.c_int
    L.rs_get_chem_kernel.argtypes = [vp, C.POINTER(i32), C.c_char_p, sz]
    L.rs_get_chem_kernel.restype = C.c_int
    L.rs_set_launch_shape.argtypes = [vp, C.c_char_p, i32]
    L.rs_set_launch_shape.restype = C.c_int
    L.rs_set_transport_staging.argtypes = [vp, i32]
    L.rs_set_transport_staging.restype = C.c_int
    L.rs_get_transport_staging.argtypes = [vp, C.POINTER(i32), C.c_char_p, sz]
    L.rs_get_transport_staging.restype = C.c_int
    L.rs_chem_kernel_source.argtypes = [C.POINTER(abi.rs_mechanism), i32, C.c_char_p, sz,
                                        C.POINTER(sz)]
    L.rs_chem_kernel_source.restype = C.c_int
    L.rs_chem_kernel_compile.argtypes = [C.POINTER(abi.rs_mechanism), i32, C.c_char_p, sz]
    L.rs_chem_kernel_compile.restype = C.c_int
    L.rs_lie_trotter_solve.argtypes = [vp, C.c_double, C.c_double, dp, dp,
                                       C.POINTER(abi.rs_solve_opts), C.POINTER(abi.rs_solve_result)]
    L.rs_lie_trotter_solve.restype = C.c_int
    L.rs_continuity_drift.argtypes = [vp, dp, dp]
    L.rs_continuity_drift.restype = C.c_int
    L.rs_lu_order.argtypes = [vp, C.POINTER(i32), i32]
    L.rs_lu_order.restype = C.c_int
    L.rs_mechanism_lu_order.argtypes = [C.POINTER(abi.rs_mechanism), i32, C.POINTER(i32), i32]
    L.rs_mechanism_lu_order.restype = C.c_int
    L.rs_chem_kernel_reciprocal.argtypes = [vp, dp, dp, sz]
    L.rs_chem_kernel_reciprocal.restype = C.c_int
    return L


def load(strict=False, build_if_missing=True, check=False):
    """Load (building in-tree if needed) the production or strict-arithmetic library, or the
    bounds-check build of the production arithmetic (check=True, built on first use)."""
    key = "check" if check else bool(strict)
    if key in _LIBS:
        return _LIBS[key]
    path = build.lib_path(strict, check)
    if check and build_if_missing:
        build.build(only=[build.CHECK_LIB])
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError("CUDA library %s is missing; run build()" % path)
        build.build()
    _LIBS[key] = _declare(C.CDLL(path))
    return _LIBS[key]


def _p(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def chem_kernel_source(mech_abi, strict=False):
    """The CUDA source generated for a mechanism's specialised chemistry kernels (no GPU)."""
    L = load(strict)
    n = C.c_size_t(0)
    rc = L.rs_chem_kernel_source(C.byref(mech_abi.struct), int(strict), None, 0, C.byref(n))
    if rc != abi.RS_OK:
        raise RsError(rc, L.rs_last_error(None).decode())
    buf = C.create_string_buffer(n.value)
    L.rs_chem_kernel_source(C.byref(mech_abi.struct), int(strict), buf, n.value, None)
    return buf.value.decode()


def mechanism_lu_order(mech_abi, natural=False):
    """The LU elimination order (species per pivot) a build uses for this mechanism: natural
    for the strict build, minimum fill for the production build.  No GPU needed."""
    L = load(False)
    n = mech_abi.struct.n_species
    ord_ = (C.c_int32 * n)()
    rc = L.rs_mechanism_lu_order(C.byref(mech_abi.struct), int(natural), ord_, n)
    if rc != abi.RS_OK:
        raise RsError(rc, L.rs_last_error(None).decode())
    return np.array(ord_[:], dtype=np.int32)


def chem_kernel_compile(mech_abi, strict=False):
    """NVRTC-compile the specialised kernels for sm_103a (no GPU); returns ptxas's report."""
    L = load(strict)
    buf = C.create_string_buffer(1 << 16)
    rc = L.rs_chem_kernel_compile(C.byref(mech_abi.struct), int(strict), buf, 1 << 16)
    if rc != abi.RS_OK:
        raise RsError(rc, L.rs_last_error(None).decode())
    return buf.value.decode()


class Solver:
    """One rs_handle: a grid + mechanism + forcing resident on the GPU."""

    def __init__(self, config, mech_abi, strict=False, check=False):
        self.L = load(strict, check=check)
        self._keep = [mech_abi]
        self.cfg = config
        h = C.c_void_p()
        rc = self.L.rs_create(C.byref(config), C.byref(h))
        if rc != abi.RS_OK:
            raise RsError(rc, self.L.rs_last_error(None).decode())
        self.h = h
        self.n = self.L.rs_state_size(h)
        self.nsp = self.L.rs_species_per_cell(h)
        g = config.grid
        self.nlon, self.nlat, self.nlev = g.nlon, g.nlat, g.nlev
        self.nc = g.nlon * g.nlat * g.nlev
        self.nr = config.mech.n_reactions

    @classmethod
    def for_workload(cls, w, strict=False, check=False, **cfg_kw):
        mabi = abi.MechanismABI(w.mech)
        s = cls(w.config(mabi, **cfg_kw), mabi, strict=strict, check=check)
        s.set_forcing(w.forcing_abi())
        return s

    def close(self):
        if getattr(self, "h", None):
            self.L.rs_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != abi.RS_OK:
            raise RsError(rc, self.L.rs_last_error(self.h).decode())

    def set_forcing(self, forcing_abi):
        self._keep.append(forcing_abi)
        self._check(self.L.rs_set_forcing(self.h, C.byref(forcing_abi.struct)))

    def set_state(self, u_cellmajor):
        u = np.ascontiguousarray(u_cellmajor, dtype=np.float64)
        self._check(self.L.rs_set_state(self.h, _p(u), u.size))

    def get_state(self, out=None):
        """The cell-major state; into `out` (float64, C-contiguous, size n) when given, e.g. a
        pinned host buffer, which the device then writes directly."""
        if out is None:
            out = np.empty(self.n)
        elif out.dtype != np.float64 or not out.flags.c_contiguous or out.size != self.n:
            raise ValueError("out must be a C-contiguous float64 array of size %d" % self.n)
        self._check(self.L.rs_get_state(self.h, _p(out), out.size))
        return out

    def rates(self):
        k = np.empty(self.nr * self.nc)
        self._check(self.L.rs_get_rate_constants(self.h, _p(k), k.size))
        return k.reshape(self.nr, self.nlev, self.nlat, self.nlon)

    def cell_steps(self):
        """Per-cell mode: (accepted substeps of each cell in the last macro step, the step
        size each cell carries), both in grid order [nlev][nlat][nlon]."""
        steps, dt = np.empty(self.nc), np.empty(self.nc)
        self._check(self.L.rs_get_cell_steps(self.h, _p(steps), _p(dt), self.nc))
        shape = (self.nlev, self.nlat, self.nlon)
        return steps.reshape(shape), dt.reshape(shape)

    def set_rates(self, k):
        k = np.ascontiguousarray(k, dtype=np.float64).reshape(-1)
        self._check(self.L.rs_set_rate_constants(self.h, _p(k), k.size))

    def macro_step(self, t0, t1, dtT, dtC, check=True):
        a, b = C.c_double(dtT), C.c_double(dtC)
        st = abi.rs_stats()
        rc = self.L.rs_macro_step(self.h, t0, t1, C.byref(a), C.byref(b), C.byref(st))
        if check:
            self._check(rc)
        return rc, a.value, b.value, st

    def rhs_transport(self, u, t=0.0):
        u = np.ascontiguousarray(u, dtype=np.float64)
        du = np.empty_like(u)
        self._check(self.L.rs_rhs_transport(self.h, t, _p(u), _p(du), u.size))
        return du

    def rhs_chem(self, u, t=0.0):
        u = np.ascontiguousarray(u, dtype=np.float64)
        du = np.empty_like(u)
        self._check(self.L.rs_rhs_chem(self.h, t, _p(u), _p(du), u.size))
        return du

    def block_jac(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64)
        J = np.empty(self.nc * self.nsp * self.nsp)
        self._check(self.L.rs_block_jac(self.h, _p(u), _p(J), J.size))
        return J.reshape(self.nc, self.nsp, self.nsp)

    def single_step(self, op, u, t, dt):
        u = np.ascontiguousarray(u, dtype=np.float64)
        un = np.empty_like(u)
        e = C.c_double()
        self._check(self.L.rs_single_step(self.h, op, t, dt, _p(u), _p(un), C.byref(e), u.size))
        return un, e.value

    # ------------------------------------------------------------ discrete adjoint
    def record(self, on=True):
        self._check(self.L.rs_record(self.h, int(on)))

    def record_count(self):
        return self.L.rs_record_count(self.h)

    def set_adjoint_tape(self, budget_bytes=-1):
        """Device-tape budget of the next recording: bytes, -1 for a quarter of the free device
        memory (the default), 0 to replay every recorded macro step from its checkpoint."""
        self._check(self.L.rs_set_adjoint_tape(self.h, int(budget_bytes)))

    def record_taped(self):
        """Recorded macro steps whose device tape is complete (swept back without replay)."""
        return self.L.rs_record_taped(self.h)

    def adjoint_backward(self, lam_end_cellmajor, steps=None, on_step=None):
        """Backward sweep over the recorded macro steps (newest first).  Returns
        (dJ/du_0 cell-major, dJ/d emission [ns][nlev][nlat][nlon])."""
        lam = np.ascontiguousarray(lam_end_cellmajor, dtype=np.float64)
        self._check(self.L.rs_adjoint_set_lambda(self.h, _p(lam), lam.size))
        self._check(self.L.rs_adjoint_reset_grad(self.h))
        n = self.record_count() if steps is None else steps
        for k in range(self.record_count() - 1, self.record_count() - 1 - n, -1):
            if on_step:
                on_step(k)
            self._check(self.L.rs_backward_macro_step(self.h, k))
        out = np.empty(self.n)
        self._check(self.L.rs_adjoint_get_lambda(self.h, _p(out), out.size))
        ns = self.cfg.mech.n_species
        g = np.empty(ns * self.nc)
        self._check(self.L.rs_adjoint_get_grad_emission(self.h, _p(g), g.size))
        return out, g.reshape(ns, self.nlev, self.nlat, self.nlon)

    def replay(self, steps=None):
        """Frozen-dt replay of the recorded macro steps 0 .. steps-1 (all by default) on the
        resident state with the forcing installed now (replay_fixed)."""
        n = self.record_count() if steps is None else steps
        for k in range(n):
            self._check(self.L.rs_replay_macro_step(self.h, k))

    def autotune(self):
        """Pick the launch shapes of this handle's kernels by timing; returns the report."""
        import json
        buf = C.create_string_buffer(16384)
        self._check(self.L.rs_autotune(self.h, buf, 16384))
        return json.loads(buf.value.decode())

    def set_chem_kernel(self, kind):
        """CHEM_KERNEL_AUTO / _TABLE / _SPECIALIZED (raises if SPECIALIZED is unavailable)."""
        self._check(self.L.rs_set_chem_kernel(self.h, int(kind)))

    def chem_kernel(self):
        """(kind in use, description dict) of the chemistry kernels."""
        import json
        k = C.c_int32(0)
        buf = C.create_string_buffer(1024)
        self._check(self.L.rs_get_chem_kernel(self.h, C.byref(k), buf, 1024))
        return k.value, json.loads(buf.value.decode())

    def set_launch_shape(self, **shape):
        """Pin launch shapes by key (the keys rs_autotune reports), e.g. mixed_yz_tracers=3."""
        for k, v in shape.items():
            self._check(self.L.rs_set_launch_shape(self.h, k.encode(), int(v)))

    def set_transport_staging(self, mode):
        """STAGING_AUTO / _PLAIN / _BULK for the mixed-precision pencils (raises if BULK is
        unavailable on this grid or precision)."""
        self._check(self.L.rs_set_transport_staging(self.h, int(mode)))

    def transport_staging(self):
        """(mode in use, per-direction description dict) of the mixed pencils' staging."""
        import json
        k = C.c_int32(0)
        buf = C.create_string_buffer(512)
        self._check(self.L.rs_get_transport_staging(self.h, C.byref(k), buf, 512))
        return k.value, json.loads(buf.value.decode())

    def lie_trotter_solve(self, t0, t1, dtT, dtC, *, macro_dt, min_macro_dt=0.0,
                          forcing_tstops=(), refresh=None, on_bisect=None):
        """One window through the library's own stop grid and bisection (rs_lie_trotter_solve)
        on the device-resident state.  Returns (status, dtT, dtC, result struct)."""
        ts = np.ascontiguousarray(np.asarray(forcing_tstops, dtype=np.float64))
        rf = abi.REFRESH_FN((lambda u, t: refresh(t)) if refresh else 0)
        bf = abi.BISECT_FN((lambda u, a, b: on_bisect(a, b)) if on_bisect else 0)
        o = abi.rs_solve_opts(float(macro_dt), float(min_macro_dt),
                              ts.ctypes.data_as(C.POINTER(C.c_double)) if ts.size else None,
                              ts.size, rf, bf, None)
        a, b = C.c_double(dtT), C.c_double(dtC)
        r = abi.rs_solve_result()
        rc = self.L.rs_lie_trotter_solve(self.h, float(t0), float(t1), C.byref(a), C.byref(b),
                                         C.byref(o), C.byref(r))
        return rc, a.value, b.value, r

    def continuity_drift(self, ps):
        """(rms over interior cells, rms over wall cells, worst interior) of (m - dp(PS))/dp(PS)."""
        ps = np.ascontiguousarray(ps, dtype=np.float64)
        out = np.zeros(3)
        self._check(self.L.rs_continuity_drift(self.h, _p(ps), _p(out)))
        return tuple(out)

    def lu_order(self):
        """Species eliminated at each pivot of this handle's LU (natural in the strict build)."""
        n = self.cfg.mech.n_species
        ord_ = (C.c_int32 * n)()
        self._check(self.L.rs_lu_order(self.h, ord_, n))
        return np.array(ord_[:], dtype=np.int32)

    def chem_kernel_reciprocal(self, x):
        """The specialised kernels' production reciprocal of each x (numerics check)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        r = np.empty_like(x)
        self._check(self.L.rs_chem_kernel_reciprocal(self.h, _p(x), _p(r), x.size))
        return r

    def stream(self):
        return self.L.rs_stream(self.h)

    def set_profiling(self, on):
        self._check(self.L.rs_set_profiling(self.h, int(on)))

    def reset_profile(self):
        self._check(self.L.rs_reset_profile(self.h))

    def profile(self):
        buf = C.create_string_buffer(4096)
        n = C.c_int32()
        la = np.zeros(64)
        ms = np.zeros(64)
        self._check(self.L.rs_get_profile(self.h, buf, 4096, _p(la), _p(ms), 64, C.byref(n)))
        names = buf.value.decode().split(";") if n.value else []
        return {nm: (la[i], ms[i]) for i, nm in enumerate(names)}
