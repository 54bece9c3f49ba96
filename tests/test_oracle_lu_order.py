"""The production build eliminates the pivot-free LU of W = I - gamma h J in a minimum-fill
order instead of the reference's natural order (the strict build keeps natural order).  The
oracle runs the reference algorithm in either order, which shows that the order changes the
reference's own results only at roundoff level on the SuperFast workloads, and within the
integration tolerance on the stiff 30-species per-cell problem (whose solution is itself only
determined to that level: one-ulp changes of dt0 move it as much)."""
import numpy as np

from reseact.esm_gb300 import abi, mechanism, workloads
from reseact.esm_gb300._lib import mechanism_lu_order


def test_natural_order_is_identity_and_min_fill_is_a_permutation():
    for m in (mechanism.superfast(), mechanism.synthetic()):
        ma = abi.MechanismABI(m)
        assert np.array_equal(mechanism_lu_order(ma, natural=True), np.arange(m.ns))
        mf = mechanism_lu_order(ma)
        assert sorted(mf.tolist()) == list(range(m.ns))
        assert not np.array_equal(mf, np.arange(m.ns))


def test_order_changes_superfast_steps_at_roundoff(oracle_lib):
    w = workloads.c1()
    mabi = abi.MechanismABI(w.mech)
    cfg = w.config(mabi)
    o = oracle_lib.Oracle(cfg, w.forcing_abi(), mabi)
    res = []
    for ordv in (None, mechanism_lu_order(mabi)):
        o.set_lu_order(ordv)
        u = np.ascontiguousarray(w.u0.copy())
        t, a, b = 0.0, 15.0, 0.5
        counts = []
        for _ in range(2):
            rc, a, b, st = o.macro_step(u, t, t + 600.0, a, b)
            counts.append(tuple(st[:4]))
            t += 600.0
        res.append((u, counts))
    (A, ca), (B, cb) = res
    assert ca == cb  # same accept/reject sequence
    rel = np.abs(B - A) / np.maximum(np.abs(A), cfg.atol_C)
    assert rel.max() < 1e-12, rel.max()


def test_order_changes_stiff_per_cell_within_tolerance(oracle_lib):
    w = workloads.c3(ncells=1024)
    mabi = abi.MechanismABI(w.mech)
    cfg = w.config(mabi)
    o = oracle_lib.Oracle(cfg, w.forcing_abi(), mabi)
    res = []
    for ordv in (None, mechanism_lu_order(mabi)):
        o.set_lu_order(ordv)
        u = np.ascontiguousarray(w.u0.copy())
        o.chem_per_cell(u, 0.0, 600.0, 1e-3)
        res.append(u)
    A, B = res
    bound = cfg.rtol_C * np.abs(A) + cfg.atol_C
    assert np.all(np.abs(B - A) <= 2.0 * bound)
    assert np.median(np.abs(B - A) / np.maximum(np.abs(A), cfg.atol_C)) < 1e-12
