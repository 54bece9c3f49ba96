"""The reference's adjoint acceptance checks on the differentiation workload, on the GPU path.

C4 is 72 x 46 x 47 with the deformational winds, SuperFast chemistry and a lognormal surface
NO emission field e; J = sum over surface cells of (O3_end - O3_obs)^2.  The library records
the macro steps (checkpoints and the accepted (t, dt) of both halves) and sweeps back; its
dJ/de is checked as the reference checks its own (tools/adjoint_gradient.jl:116-132):

* fdtape: central differences, h = 1e-6 relative, of the FROZEN-dt composed map (every
  recorded macro step replayed with its recorded step sequence, rs_replay_macro_step) at 20
  seeded surface cells;
* ident: scaling the whole field, d J(s e) / ds at s = 1 equals <e, dJ/de>;
* the clamp switched off (the reference's adjoint demo runs with RESEACT_ADJ_CLAMP=0,
  run_reseact_adjoint.jl:400): the sweep still matches the oracle's.
"""
import numpy as np
import pytest

from reseact.esm_gb300 import Solver, abi, workloads

pytestmark = pytest.mark.gpu

STEPS = 12  # two hours of the 24 h window: 12 recorded macro steps of 600 s


def _objective(w, u_cm, obs, iO3):
    g = w.grid
    u = workloads.cellmajor_to_soa(u_cm, w.nsp, g["nlon"], g["nlat"], g["nlev"])
    return float(np.sum((u[iO3, 0] - obs) ** 2)), u


@pytest.fixture(scope="module")
def c4_recorded():
    w = workloads.c4()
    g = w.grid
    iNO, iO3 = w.mech.species.index("NO"), w.mech.species.index("O3")
    obs = 30.0 * np.exp(0.3 * np.random.default_rng(44).standard_normal((g["nlat"], g["nlon"])))
    s = Solver.for_workload(w)
    s.set_state(w.u0_cellmajor())
    s.record(True)
    t, a, b = 0.0, w.dt0_T, w.dt0_C
    for _ in range(STEPS):
        _, a, b, _ = s.macro_step(t, t + w.dt_macro, a, b)
        t += w.dt_macro
    s.record(False)
    J0, uend = _objective(w, s.get_state(), obs, iO3)
    lam = np.zeros_like(uend)
    lam[iO3, 0] = 2 * (uend[iO3, 0] - obs)
    _, grad = s.adjoint_backward(workloads.soa_to_cellmajor(lam, g["nlon"], g["nlat"], g["nlev"]))
    return w, s, obs, iNO, iO3, J0, grad[iNO, 0]


def _replayed_J(w, s, obs, iO3, emis_surface, iNO):
    """J of the frozen-dt map from the initial state with the given surface NO emission."""
    e = np.array(w.forcing["emission"])
    e[iNO, 0] = emis_surface
    s.set_forcing(abi.ForcingABI(emission=e))
    s.set_state(w.u0_cellmajor())
    s.replay()
    return _objective(w, s.get_state(), obs, iO3)[0]


def test_replay_reproduces_the_recorded_forward(c4_recorded):
    """The frozen-dt replay at the unperturbed forcing lands on the forward's end state."""
    w, s, obs, iNO, iO3, J0, _ = c4_recorded
    e0 = np.array(w.forcing["emission"])[iNO, 0]
    assert _replayed_J(w, s, obs, iO3, e0, iNO) == pytest.approx(J0, rel=1e-13)


def test_fdtape_central_differences_at_20_surface_cells(c4_recorded):
    w, s, obs, iNO, iO3, J0, g = c4_recorded
    e0 = np.array(w.forcing["emission"])[iNO, 0]
    rng = np.random.default_rng(20)
    nlat, nlon = e0.shape
    cells = [(int(j), int(i)) for j, i in zip(rng.integers(0, nlat, 20), rng.integers(0, nlon, 20))]
    h = 1e-6
    fd, ad = [], []
    for j, i in cells:
        d = h * e0[j, i]
        ep, em = e0.copy(), e0.copy()
        ep[j, i] += d
        em[j, i] -= d
        Jp = _replayed_J(w, s, obs, iO3, ep, iNO)
        Jm = _replayed_J(w, s, obs, iO3, em, iNO)
        fd.append((Jp - Jm) / (2 * d))
        ad.append(g[j, i])
    fd, ad = np.array(fd), np.array(ad)
    scale = np.abs(ad).max()
    assert scale > 0
    err = np.abs(fd - ad) / np.maximum(np.abs(ad), 1e-3 * scale)
    assert err.max() < 1e-4, list(zip(cells, fd, ad, err))


def test_ident_scaling_identity(c4_recorded):
    """d J(s e) / ds at s = 1 (central differences of the frozen-dt map, h = 1e-6) equals
    <e, dJ/de> from the adjoint."""
    w, s, obs, iNO, iO3, J0, g = c4_recorded
    e0 = np.array(w.forcing["emission"])[iNO, 0]
    h = 1e-6
    dJds = (_replayed_J(w, s, obs, iO3, (1 + h) * e0, iNO)
            - _replayed_J(w, s, obs, iO3, (1 - h) * e0, iNO)) / (2 * h)
    ident = float(np.sum(e0 * g))
    assert dJds == pytest.approx(ident, rel=1e-5), (dJds, ident)


@pytest.fixture(scope="module")
def oracle_mod():
    from oracle import oracle
    oracle.build()
    return oracle


def test_sweep_with_clamp_off_matches_oracle(oracle_mod):
    """clamp_nonneg = 0, the reference's adjoint demo setting: the GPU sweep over three
    recorded macro steps matches the oracle's (itself checked against finite differences)."""
    rng = np.random.default_rng(3)
    w = workloads.c2(nlon=12, nlat=9, nlev=6)
    g = w.grid
    iNO, iO3 = w.mech.species.index("NO"), w.mech.species.index("O3")
    emis = np.zeros((w.mech.ns, g["nlev"], g["nlat"], g["nlon"]))
    emis[iNO, 0] = 1e-4 * np.exp(0.5 * rng.standard_normal((g["nlat"], g["nlon"])))
    w.forcing["emission"] = emis
    obs = 30.0 * np.exp(0.3 * rng.standard_normal((g["nlat"], g["nlon"])))
    mabi = abi.MechanismABI(w.mech)
    cfg = w.config(mabi, clamp_nonneg=False)
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
        assert orc == 0 and (st.naT, st.naC) == (ost[0], ost[2])
        t += 600.0
    s.record(False)
    uend = workloads.cellmajor_to_soa(s.get_state(), w.nsp, g["nlon"], g["nlat"], g["nlev"])
    lam = np.zeros_like(uend)
    lam[iO3, 0] = 2 * (uend[iO3, 0] - obs)
    lg, eg = s.adjoint_backward(workloads.soa_to_cellmajor(lam, g["nlon"], g["nlat"], g["nlev"]))
    lo, eo = o.adjoint_backward(lam)
    lo = workloads.soa_to_cellmajor(lo, g["nlon"], g["nlat"], g["nlev"])
    scale = np.abs(lo).max()
    assert np.abs(lg - lo).max() <= 1e-8 * scale, np.abs(lg - lo).max() / scale
    e_g, e_o = eg[iNO, 0], eo[iNO, 0]
    assert np.abs(e_g - e_o).max() <= 1e-8 * np.abs(e_o).max()
