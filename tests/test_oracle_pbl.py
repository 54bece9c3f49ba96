"""Full PBL mixing (reseact.esm Transport3D: pbl_f, pbl_wt, pbl_mean_*, tendency
pbl_f*(pbl_mean - q)/tau_pblmix) in the oracle: the invariants the reference states for it
(exact column mass conservation; relaxation to the PBL mean) and its transport-RHS VJP
against central finite differences."""
import numpy as np

from reseact.esm_gb300 import abi, workloads


def _still(w):
    """No advection: only the PBL term moves tracers."""
    for k in ("mx", "my", "mz"):
        w.forcing[k] = np.zeros_like(w.forcing[k])
    return w


def _oracle(oracle_lib, w, **kw):
    mabi = abi.MechanismABI(w.mech)
    cfg = w.config(mabi, **kw)
    return oracle_lib.Oracle(cfg, w.forcing_abi(), mabi), cfg


def test_pbl_term_conserves_column_mass(oracle_lib):
    w = workloads.with_pbl(_still(workloads.c2(nlon=12, nlat=7, nlev=12, steps=1)), tau=300.0,
                           pblh_median=2500.0)
    o, _ = _oracle(oracle_lib, w, do_chemistry=False)
    du = o.rhs_transport(np.ascontiguousarray(w.u0))
    dp = np.asarray(w.forcing["dp"])
    ntr = w.mech.ns
    assert np.abs(du[:ntr]).max() > 0  # the term acts
    col = (du[:ntr] * dp[None]).sum(axis=1)          # sum_k dp_k d(q_k)/dt per tracer, column
    scale = (np.abs(du[:ntr]) * dp[None]).sum(axis=1)
    assert np.all(np.abs(col) <= 1e-13 * scale + 1e-300)
    # layers wholly above the PBL top (lower interface pressure <= p_top) are untouched
    f = w.forcing
    ptop = f["ps"] * np.exp(-(f["pblh"] * 9.80665) / (287.05 * f["temperature"][0]))
    above = f["hyb_a"][:-1, None, None] <= ptop[None]
    assert above.any() and np.all(du[:ntr][:, above] == 0.0)


def test_pbl_relaxes_profile_to_its_mean(oracle_lib):
    w = workloads.with_pbl(_still(workloads.c2(nlon=8, nlat=5, nlev=12, steps=1)), tau=60.0,
                           pblh_median=2500.0, sigma=0.0)
    o, cfg = _oracle(oracle_lib, w, do_chemistry=False)
    u = np.ascontiguousarray(w.u0.copy())
    dp = np.asarray(w.forcing["dp"])
    ntr = w.mech.ns
    m0 = (u[:ntr] * dp[None]).sum(axis=1)
    rc, _, _, _ = o.macro_step(u, 0.0, 1800.0, 15.0, 0.5)  # 30 relaxation times
    assert rc == 0
    assert np.allclose((u[:ntr] * dp[None]).sum(axis=1), m0, rtol=1e-12, atol=0)
    # layers wholly inside the PBL (lowest two) end at one common value per column
    inside = u[:ntr, :2]
    spread = np.abs(inside[:, 0] - inside[:, 1]) / np.abs(inside).max(axis=1)
    assert spread.max() < 1e-6


def test_pbl_transport_vjp_matches_finite_differences(oracle_lib):
    rng = np.random.default_rng(3)
    w = workloads.with_pbl(workloads.c2(nlon=8, nlat=5, nlev=10, steps=1), tau=500.0,
                           pblh_median=2500.0)
    o, _ = _oracle(oracle_lib, w, do_chemistry=False)
    u = np.ascontiguousarray(w.u0.copy())
    fbar = rng.standard_normal(u.shape)
    ubar = o.transport_rhs_vjp(u, 0.0, fbar)
    for _ in range(6):
        d = rng.standard_normal(u.shape) * np.abs(u) * 1e-3
        h = 1e-3
        fp = o.rhs_transport(np.ascontiguousarray(u + h * d))
        fm = o.rhs_transport(np.ascontiguousarray(u - h * d))
        fd = np.sum(fbar * (fp - fm)) / (2 * h)
        assert abs(np.sum(ubar * d) - fd) <= 1e-6 * abs(fd) + 1e-12, (np.sum(ubar * d), fd)
