"""The oracle's discrete adjoint, pinned by central finite differences on the CPU.

Mirrors the reference's checks (tools/rx_adjoint_check.jl: FD sweep of one step's VJP;
tools/adjoint_gradient.jl `fdtape`: central FD of the frozen-dt composed map) at a jittered,
non-uniform base point (PPM limiters are not differentiable on uniform fields,
tools/diag/ppm_limiter_kink_repro.jl).  The objective is the C4 one: J = sum over surface
cells of (O3_end - O3_obs)^2, gradient w.r.t. a surface NO emission field."""
import numpy as np
import pytest

from reseact.esm_gb300 import abi, workloads


def _setup(oracle_lib, do_T=True, do_C=True, seed=1):
    rng = np.random.default_rng(seed)
    w = workloads.c2(nlon=12, nlat=9, nlev=6)
    g = w.grid
    iNO, iO3 = w.mech.species.index("NO"), w.mech.species.index("O3")
    emis = np.zeros((w.mech.ns, g["nlev"], g["nlat"], g["nlon"]))
    emis[iNO, 0] = 1e-4 * np.exp(0.5 * rng.standard_normal((g["nlat"], g["nlon"])))
    w.forcing["emission"] = emis
    mabi = abi.MechanismABI(w.mech)
    cfg = w.config(mabi, do_transport=do_T, do_chemistry=do_C)
    o = oracle_lib.Oracle(cfg, w.forcing_abi(), mabi)
    return w, o, emis, iNO, iO3, rng, mabi


def test_step_vjps_match_central_fd(oracle_lib):
    w, o, emis, iNO, iO3, rng, _ = _setup(oracle_lib)
    u = np.ascontiguousarray(w.u0.copy())
    lam = rng.standard_normal(u.shape)
    v = rng.standard_normal(u.shape) * np.abs(u) * 1e-3
    t = 1000.0
    eps = 1e-3
    # transport RHS
    ub = o.transport_rhs_vjp(u, t, lam)
    fd = np.sum(lam * (o.rhs_transport(u + eps * v, t) - o.rhs_transport(u - eps * v, t))) / (2 * eps)
    assert np.sum(ub * v) == pytest.approx(fd, rel=1e-7)
    # one SSPRK43 step
    lb = o.ssprk43_vjp(u, t, 200.0, lam)
    up, _ = o.single_step(abi.RS_OP_TRANSPORT, u + eps * v, t, 200.0)
    um, _ = o.single_step(abi.RS_OP_TRANSPORT, u - eps * v, t, 200.0)
    assert np.sum(lb * v) == pytest.approx(np.sum(lam * (up - um)) / (2 * eps), rel=1e-8)
    # one ROS23 step (air mass is inert in chemistry)
    vc = rng.standard_normal(u.shape) * np.abs(u) * 1e-4
    vc[-1] = 0
    lc, eb = o.ros23_vjp(u, 30.0, lam)
    up, _ = o.single_step(abi.RS_OP_CHEMISTRY, u + 1e-2 * vc, t, 30.0)
    um, _ = o.single_step(abi.RS_OP_CHEMISTRY, u - 1e-2 * vc, t, 30.0)
    assert np.sum(lc * vc) == pytest.approx(np.sum(lam * (up - um)) / 2e-2, rel=1e-8)


@pytest.mark.parametrize("do_T", [True, False])
def test_emission_gradient_matches_fixed_sequence_fd(oracle_lib, do_T):
    w, o, emis, iNO, iO3, rng, _ = _setup(oracle_lib, do_T=do_T)
    g = w.grid
    u0 = np.ascontiguousarray(w.u0.copy())
    u = u0.copy()
    obs = 30.0 * np.exp(0.3 * rng.standard_normal((g["nlat"], g["nlon"])))
    t, dtT, dtC = 0.0, 15.0, 0.5
    for _ in range(3):
        rc, dtT, dtC, _ = o.record_macro_step(u, t, t + 600.0, dtT, dtC)
        assert rc == 0
        t += 600.0
    assert np.array_equal(o.replay(u0), u)  # the fixed-sequence replay IS the forward
    J = lambda ue: np.sum((ue[iO3, 0] - obs) ** 2)
    lam = np.zeros_like(u)
    lam[iO3, 0] = 2 * (u[iO3, 0] - obs)
    l0, eb = o.adjoint_backward(lam)
    for (j, i) in [(2, 3), (5, 7), (7, 1), (4, 10)]:
        h = 1e-4 * emis[iNO, 0, j, i]
        ep, em = emis.copy(), emis.copy()
        ep[iNO, 0, j, i] += h
        em[iNO, 0, j, i] -= h
        o.set_forcing(abi.ForcingABI(emission=ep))
        Jp = J(o.replay(u0))
        o.set_forcing(abi.ForcingABI(emission=em))
        Jm = J(o.replay(u0))
        fd = (Jp - Jm) / (2 * h)
        assert eb[iNO, 0, j, i] == pytest.approx(fd, rel=1e-6)
    # initial-state gradient of the surface O3 field
    o.set_forcing(abi.ForcingABI(emission=emis))
    idx = (iO3, 0, 4, 4)
    h = 1e-4 * u0[idx]
    up, um = u0.copy(), u0.copy()
    up[idx] += h
    um[idx] -= h
    fd = (J(o.replay(up)) - J(o.replay(um))) / (2 * h)
    assert l0[idx] == pytest.approx(fd, rel=1e-6)
