"""GPU discrete adjoint against the oracle's (itself pinned by central finite differences in
tests/test_oracle_adjoint.py), through the C ABI: record three macro steps, sweep back with
lambda_end = dJ/du_end of the C4 objective J = sum_surface (O3_end - O3_obs)^2, compare
dJ/du_0 and dJ/d(surface NO emission)."""
import numpy as np
import pytest

from reseact.esm_gb300 import Solver, abi, workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def oracle_mod():
    from oracle import oracle
    oracle.build()
    return oracle


def _case(do_T=True, do_C=True, seed=1):
    rng = np.random.default_rng(seed)
    w = workloads.c2(nlon=12, nlat=9, nlev=6)
    g = w.grid
    iNO, iO3 = w.mech.species.index("NO"), w.mech.species.index("O3")
    emis = np.zeros((w.mech.ns, g["nlev"], g["nlat"], g["nlon"]))
    emis[iNO, 0] = 1e-4 * np.exp(0.5 * rng.standard_normal((g["nlat"], g["nlon"])))
    w.forcing["emission"] = emis
    obs = 30.0 * np.exp(0.3 * rng.standard_normal((g["nlat"], g["nlon"])))
    return w, iNO, iO3, obs, dict(do_transport=do_T, do_chemistry=do_C)


@pytest.mark.parametrize("do_T,do_C", [(True, True), (True, False), (False, True)])
def test_adjoint_sweep_matches_oracle(oracle_mod, do_T, do_C):
    w, iNO, iO3, obs, kw = _case(do_T, do_C)
    g = w.grid
    mabi = abi.MechanismABI(w.mech)
    cfg = w.config(mabi, **kw)
    s = Solver(cfg, mabi)
    f = w.forcing_abi()
    s.set_forcing(f)
    o = oracle_mod.Oracle(cfg, f, mabi)
    o.set_lu_order(s.lu_order())
    o.set_rates(s.rates())
    s.set_state(w.u0_cellmajor())
    s.record(True)
    u = np.ascontiguousarray(w.u0.copy())
    t, a, b, ao, bo = 0.0, 15.0, 0.5, 15.0, 0.5
    for _ in range(3):
        _, a, b, st = s.macro_step(t, t + 600.0, a, b)
        orc, ao, bo, ost = o.record_macro_step(u, t, t + 600.0, ao, bo)
        assert (st.naT, st.naC) == (ost[0], ost[2])
        t += 600.0
    s.record(False)
    assert s.record_count() == 3
    uend = workloads.cellmajor_to_soa(s.get_state(), w.nsp, g["nlon"], g["nlat"], g["nlev"])
    lam = np.zeros_like(uend)
    lam[iO3, 0] = 2 * (uend[iO3, 0] - obs)
    lg, eg = s.adjoint_backward(workloads.soa_to_cellmajor(lam, g["nlon"], g["nlat"], g["nlev"]))
    lo, eo = o.adjoint_backward(lam)
    lo = workloads.soa_to_cellmajor(lo, g["nlon"], g["nlat"], g["nlev"])
    scale = np.abs(lo).max()
    assert np.abs(lg - lo).max() <= 1e-8 * scale, np.abs(lg - lo).max() / scale
    if do_C:
        e_g, e_o = eg[iNO, 0], eo[iNO, 0]
        assert np.abs(e_g - e_o).max() <= 1e-8 * np.abs(e_o).max()
        assert np.abs(e_o).max() > 0
    # deterministic: a second sweep gives the same bits
    lg2, eg2 = s.adjoint_backward(workloads.soa_to_cellmajor(lam, g["nlon"], g["nlat"], g["nlev"]))
    assert np.array_equal(lg, lg2) and np.array_equal(eg, eg2)


def test_backward_requires_recording():
    w, iNO, iO3, obs, kw = _case()
    s = Solver.for_workload(w)
    from reseact.esm_gb300._lib import RsError
    with pytest.raises(RsError):
        s.adjoint_backward(np.zeros(s.n), steps=1)


def _sweep(w, iO3, obs, kw, budget):
    """Record three macro steps with the given device-tape budget, sweep back; returns the
    gradients and the number of macro steps swept from the tape."""
    g = w.grid
    s = Solver.for_workload(w, **kw)
    s.set_adjoint_tape(budget)
    s.set_state(w.u0_cellmajor())
    s.record(True)
    t, a, b = 0.0, 15.0, 0.5
    for _ in range(3):
        _, a, b, _ = s.macro_step(t, t + 600.0, a, b)
        t += 600.0
    s.record(False)
    uend = workloads.cellmajor_to_soa(s.get_state(), w.nsp, g["nlon"], g["nlat"], g["nlev"])
    lam = np.zeros_like(uend)
    lam[iO3, 0] = 2 * (uend[iO3, 0] - obs)
    lg, eg = s.adjoint_backward(workloads.soa_to_cellmajor(lam, g["nlon"], g["nlat"], g["nlev"]))
    taped = s.record_taped()
    s.close()
    return lg, eg, taped


def test_device_tape_equals_replay_bitwise():
    """The forward's device tape (every accepted step's input, chemistry stages and transport
    stage records kept in HBM) and the replay from checkpoints give the same gradients bit for
    bit -- the replay reproduces the forward's states and stages exactly -- whether all, none
    or only the first recorded macro steps fit the tape."""
    w, iNO, iO3, obs, kw = _case()
    lg, eg, taped = _sweep(w, iO3, obs, kw, -1)
    assert taped == 3
    lr, er, taped0 = _sweep(w, iO3, obs, kw, 0)
    assert taped0 == 0
    assert np.array_equal(lg, lr) and np.array_equal(eg, er)
    # room for the first macro step and half of another: the first is taped, the rest replay.
    # A macro step needs its states (nsp doubles per cell, one per step and the end state), the
    # chemistry stages k1, z2 (2 ns per cell and chemistry step) and the transport stage
    # records (7 nsp per cell and transport step); the three share the budget in fixed
    # proportions close to these
    nc = w.grid["nlon"] * w.grid["nlat"] * w.grid["nlev"]
    s = Solver.for_workload(w, **kw)
    s.set_state(w.u0_cellmajor())
    s.record(True)
    st = s.macro_step(0.0, 600.0, 15.0, 0.5)[3]
    s.close()
    nT, nC = int(st.naT), int(st.naC)
    need = ((nT + nC + 1) * w.nsp + nC * 2 * w.mech.ns + nT * 7 * w.nsp) * nc * 8
    lp, ep, tapedp = _sweep(w, iO3, obs, kw, int(1.5 * need))
    assert tapedp == 1
    assert np.array_equal(lg, lp) and np.array_equal(eg, ep)
