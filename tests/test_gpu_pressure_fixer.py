"""Pressure fixer with diagnosed vertical mass flux on the GPU (the second next row,
reseact.esm Transport3D divh_fix / Mz / dm/dt) against the oracle through the C ABI, and the
continuity drift diagnostic of run_reseact.jl:297-324."""
import numpy as np
import pytest

from reseact.esm_gb300 import Solver, abi, workloads
from reseact.esm_gb300._lib import RsError

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def oracle_mod():
    from oracle import oracle
    oracle.build()
    return oracle


def _w():
    return workloads.with_pressure_fixer(workloads.c2(nlon=16, nlat=9, nlev=12, steps=1))


def _pair(w, oracle_mod, strict=False, **kw):
    mabi = abi.MechanismABI(w.mech)
    cfg = w.config(mabi, **kw)
    s = Solver(cfg, mabi, strict=strict)
    f = w.forcing_abi()
    s.set_forcing(f)
    o = oracle_mod.Oracle(cfg, f, mabi)
    o.set_lu_order(s.lu_order())
    o.set_rates(s.rates())
    return s, o


def cm(w, u):
    g = w.grid
    return workloads.soa_to_cellmajor(u, g["nlon"], g["nlat"], g["nlev"])


@pytest.mark.parametrize("strict", [False, True])
def test_transport_rhs_with_fixer(oracle_mod, strict):
    w = _w()
    s, o = _pair(w, oracle_mod, strict=strict)
    du_o = cm(w, o.rhs_transport(w.u0, 0.0))
    du_g = s.rhs_transport(w.u0_cellmajor(), 0.0)
    if strict:
        assert np.array_equal(du_g, du_o)
    else:
        scale = np.abs(du_o).reshape(-1, w.nsp).max(axis=0)
        err = np.abs(du_g - du_o).reshape(-1, w.nsp) / scale
        assert err.max() < 1e-12, err.max()
    # continuity identity on the device: dm_k/dt == dB_k dPS/dt
    f = w.forcing
    g = w.grid
    dm = workloads.cellmajor_to_soa(du_g, w.nsp, g["nlon"], g["nlat"], g["nlev"])[-1]
    want = (f["hyb_b"][:-1] - f["hyb_b"][1:])[:, None, None] * f["dps_dt"][None]
    assert (np.abs(dm - want) / np.asarray(f["dp"])).max() < 1e-17


@pytest.mark.parametrize("precision", [abi.RS_PREC_FP64, abi.RS_PREC_MIXED])
def test_macro_steps_with_fixer(oracle_mod, precision):
    """FP64 and the compensated FP32 transport (face fluxes, the diagnosed Mz included, as
    float pairs; the air-mass row and its fixer correction in FP64) against the FP64 oracle."""
    w = _w()
    s, o = _pair(w, oracle_mod, precision=precision)
    s.set_state(w.u0_cellmajor())
    u = np.ascontiguousarray(w.u0.copy())
    a_g = a_o = 15.0
    b_g = b_o = 0.5
    t = 0.0
    for _ in range(3):
        rc, a_g, b_g, st = s.macro_step(t, t + 600.0, a_g, b_g)
        orc, a_o, b_o, ost = o.macro_step(u, t, t + 600.0, a_o, b_o)
        assert orc == 0 and (st.naT, st.nrT, st.naC, st.nrC) == tuple(ost[:4])
        t += 600.0
    got, ref = s.get_state(), cm(w, u)
    err = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-9)
    assert err.max() < 1e-10, err.max()
    # the air mass follows dp(PS(t)); the continuity diagnostic sees no drift
    f = w.forcing
    rms_int, rms_wall, worst = s.continuity_drift(f["ps"] + f["dps_dt"] * t)
    assert rms_int < 1e-13 and rms_wall < 1e-13 and abs(worst) < 1e-13


def test_drift_without_the_fixer_is_seen():
    w = workloads.c2(nlon=16, nlat=9, nlev=12, steps=1)
    wf = _w()
    w.forcing["flux_omega"] = 0.0
    w.forcing["hyb_a"], w.forcing["hyb_b"] = wf.forcing["hyb_a"], wf.forcing["hyb_b"]
    s = Solver.for_workload(w, do_chemistry=False)
    s.set_state(w.u0_cellmajor())
    s.macro_step(0.0, 1800.0, 15.0, 0.5)
    rms_int, _, worst = s.continuity_drift(np.full((9, 16), wf.forcing["ps"][0, 0]))
    assert rms_int > 1e-6


def test_fixer_needs_steady_fluxes():
    w = workloads.c2(nlon=16, nlat=9, nlev=12, steps=1)  # flux_omega = pi/86400
    wf = _w()
    for k in ("hyb_a", "hyb_b", "dps_dt"):
        w.forcing[k] = wf.forcing[k]
    with pytest.raises(RsError) as e:
        Solver.for_workload(w)
    assert e.value.status == abi.RS_ERR_UNSUPPORTED


def test_adjoint_with_fixer_matches_oracle_taped_or_replayed(oracle_mod):
    """The discrete adjoint with the pressure fixer (its correction enters the air-mass
    tendency but not the state derivative) against the oracle, with the device tape and with
    the replay -- the transport stage records carry the corrected air-mass tendency."""
    w = _w()
    g = w.grid
    iO3 = w.mech.species.index("O3")
    grads = []
    for budget in (-1, 0):
        s, o = _pair(w, oracle_mod)
        s.set_adjoint_tape(budget)
        s.set_state(w.u0_cellmajor())
        s.record(True)
        u = np.ascontiguousarray(w.u0.copy())
        t, a, b, ao, bo = 0.0, 15.0, 0.5, 15.0, 0.5
        for _ in range(2):
            _, a, b, st = s.macro_step(t, t + 600.0, a, b)
            orc, ao, bo, ost = o.record_macro_step(u, t, t + 600.0, ao, bo)
            assert (st.naT, st.naC) == (ost[0], ost[2])
            t += 600.0
        s.record(False)
        assert s.record_taped() == (2 if budget else 0)
        uend = workloads.cellmajor_to_soa(s.get_state(), w.nsp, g["nlon"], g["nlat"], g["nlev"])
        lam = np.zeros_like(uend)
        lam[iO3, 0] = 2 * uend[iO3, 0]
        lg, _ = s.adjoint_backward(cm(w, lam))
        lo, _ = o.adjoint_backward(lam)
        lo = cm(w, lo)
        scale = np.abs(lo).max()
        assert np.abs(lg - lo).max() <= 1e-8 * scale, np.abs(lg - lo).max() / scale
        grads.append(lg)
        s.close()
    assert np.array_equal(grads[0], grads[1])
