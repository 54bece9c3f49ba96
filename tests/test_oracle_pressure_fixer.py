"""Pressure fixer with diagnosed vertical mass flux (reseact.esm Transport3D divh_fix, Mz,
dm/dt) in the oracle: the continuity identity the reference pins, dm_k/dt == dB_k dPS/dt to
roundoff (its metadata quotes ~1e-17 s^-1 relative to dp); the exact CWC freestream with the
diagnosed Mz; and no drift of m against dp(PS(t)) over adaptive steps."""
import numpy as np

from reseact.esm_gb300 import abi, workloads


def _w():
    return workloads.with_pressure_fixer(workloads.c2(nlon=12, nlat=9, nlev=12, steps=1))


def _oracle(oracle_lib, w, **kw):
    mabi = abi.MechanismABI(w.mech)
    cfg = w.config(mabi, **kw)
    return oracle_lib.Oracle(cfg, w.forcing_abi(), mabi), cfg


def test_continuity_identity(oracle_lib):
    w = _w()
    o, _ = _oracle(oracle_lib, w, do_chemistry=False)
    du = o.rhs_transport(np.ascontiguousarray(w.u0))
    f = w.forcing
    dB = f["hyb_b"][:-1] - f["hyb_b"][1:]
    want = dB[:, None, None] * f["dps_dt"][None]
    dp = np.asarray(f["dp"])
    resid = np.abs(du[-1] - want) / dp
    assert resid.max() < 1e-17, resid.max()
    # without the fixer the same fluxes move the air mass by the raw divergence
    w0 = workloads.c2(nlon=12, nlat=9, nlev=12, steps=1)
    w0.forcing["flux_omega"] = 0.0
    o0, _ = _oracle(oracle_lib, w0, do_chemistry=False)
    du0 = o0.rhs_transport(np.ascontiguousarray(w0.u0))
    assert (np.abs(du0[-1] - want) / dp).max() > 1e-9


def test_freestream_stays_exact_with_diagnosed_mz(oracle_lib):
    w = _w()
    u = np.ascontiguousarray(w.u0.copy())
    u[:-1] = 1.0
    o, _ = _oracle(oracle_lib, w, do_chemistry=False)
    du = o.rhs_transport(u)
    assert np.all(du[:-1] == 0.0)


def test_air_mass_follows_surface_pressure(oracle_lib):
    w = _w()
    o, _ = _oracle(oracle_lib, w, do_chemistry=False)
    u = np.ascontiguousarray(w.u0.copy())
    rc, _, _, _ = o.macro_step(u, 0.0, 1800.0, 15.0, 0.5)
    assert rc == 0
    f = w.forcing
    ps = f["ps"] + f["dps_dt"] * 1800.0
    dpk = (f["hyb_a"][:-1] - f["hyb_a"][1:])[:, None, None] + \
          (f["hyb_b"][:-1] - f["hyb_b"][1:])[:, None, None] * ps[None]
    r = (u[-1] - dpk) / dpk
    assert np.abs(r).max() < 1e-13, np.abs(r).max()
