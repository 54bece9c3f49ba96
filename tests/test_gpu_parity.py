"""GPU parity against the CPU oracle, through the C ABI.

Two builds are checked: the strict one (--fmad=false, divides where the reference divides)
must reproduce the oracle BIT FOR BIT given the same rate constants; the production build
(FMA contraction, reciprocal multiplies) must agree to the spec FP64 tolerance,
relative 1e-10 (with the solver's absolute tolerance as the floor for values near zero).
Sizes are small so the oracle finishes in seconds.
"""
import numpy as np
import pytest

from reseact.esm_gb300 import Solver, abi, workloads
from reseact.esm_gb300._lib import RsError

from parity_util import per_cell_agreement

pytestmark = pytest.mark.gpu

REL = 1e-10  # spec FP64 parity tolerance


@pytest.fixture(scope="module")
def oracle_mod():
    from oracle import oracle
    oracle.build()
    return oracle


def small_c2(nlon=16, nlat=9, nlev=6, seed=2):
    return workloads.c2(seed=seed, nlon=nlon, nlat=nlat, nlev=nlev, steps=1)


def small_c1(seed=1):
    w = workloads.c1(seed=seed)
    return w


def make_pair(w, oracle_mod, strict=False, **kw):
    mabi = abi.MechanismABI(w.mech)
    cfg = w.config(mabi, **kw)
    s = Solver(cfg, mabi, strict=strict)
    f = w.forcing_abi()
    s.set_forcing(f)
    o = oracle_mod.Oracle(cfg, f, mabi)
    o.set_lu_order(s.lu_order())  # the handle's elimination order
    return s, o


def cm(w, u):
    g = w.grid
    return workloads.soa_to_cellmajor(u, g["nlon"], g["nlat"], g["nlev"])


def close(a, b, rel=REL, floor=0.0):
    a, b = np.asarray(a), np.asarray(b)
    err = np.abs(a - b)
    lim = rel * np.maximum(np.abs(b), floor)
    return bool(np.all(err <= lim)), float(np.max(err / np.maximum(np.maximum(np.abs(b), floor), 1e-300)))


def test_state_roundtrip_is_exact(oracle_mod):
    w = small_c2()
    s, _ = make_pair(w, oracle_mod)
    u = w.u0_cellmajor()
    s.set_state(u)
    assert np.array_equal(s.get_state(), u)


@pytest.mark.parametrize("strict", [False, True])
def test_rate_constants_match_oracle(oracle_mod, strict):
    w = small_c2()
    s, o = make_pair(w, oracle_mod, strict=strict)
    kg, ko = s.rates(), o.rates()
    ok, worst = close(kg, ko, rel=2e-15)
    assert ok, worst


@pytest.mark.parametrize("strict", [False, True])
def test_chem_rhs_and_jacobian(oracle_mod, strict):
    w = small_c2()
    s, o = make_pair(w, oracle_mod, strict=strict)
    o.set_rates(s.rates())  # same k on both sides
    u = w.u0
    du_o = cm(w, o.rhs_chem(u))
    du_g = s.rhs_chem(cm(w, u))
    J_o = o.block_jac(u)
    J_g = s.block_jac(cm(w, u))
    # oracle J is in grid-cell order; reorder to the cell-major cell index
    g = w.grid
    order = np.arange(w.ncells).reshape(g["nlev"], g["nlat"], g["nlon"]).transpose(2, 1, 0).reshape(-1)
    J_o = J_o[order]
    if strict:
        assert np.array_equal(du_g, du_o)
        assert np.array_equal(J_g, J_o)
    else:
        scale = np.abs(du_o).reshape(-1, w.nsp).max(axis=0)
        ok, worst = close(du_g.reshape(-1, w.nsp), du_o.reshape(-1, w.nsp), rel=1e-12,
                          floor=1e-3 * scale.max())
        assert ok, worst
        assert np.allclose(J_g, J_o, rtol=1e-13, atol=1e-13 * np.abs(J_o).max())


@pytest.mark.parametrize("strict", [False, True])
def test_transport_rhs(oracle_mod, strict):
    w = small_c2()
    s, o = make_pair(w, oracle_mod, strict=strict)
    for t in (0.0, 3600.0):
        du_o = cm(w, o.rhs_transport(w.u0, t))
        du_g = s.rhs_transport(w.u0_cellmajor(), t)
        if strict:
            assert np.array_equal(du_g, du_o)
        else:
            scale = np.abs(du_o).reshape(-1, w.nsp).max(axis=0)
            err = np.abs(du_g - du_o).reshape(-1, w.nsp) / scale
            assert err.max() < 1e-12, err.max()


@pytest.mark.parametrize("strict", [False, True])
@pytest.mark.parametrize("op", [abi.RS_OP_TRANSPORT, abi.RS_OP_CHEMISTRY])
def test_single_step(oracle_mod, strict, op):
    w = small_c1()  # steady fluxes: stage factors are exactly 1 on both sides
    s, o = make_pair(w, oracle_mod, strict=strict)
    o.set_rates(s.rates())
    dt = 120.0 if op == abi.RS_OP_TRANSPORT else 2.0
    un_o, e_o = o.single_step(op, w.u0, 0.0, dt)
    un_g, e_g = s.single_step(op, w.u0_cellmajor(), 0.0, dt)
    if strict:
        assert np.array_equal(un_g, cm(w, un_o))
        assert e_g == e_o
    else:
        ok, worst = close(un_g, cm(w, un_o), rel=1e-12, floor=1e-9)
        assert ok, worst
        assert e_g == pytest.approx(e_o, rel=1e-10)


@pytest.mark.parametrize("wname", ["c1", "c2"])
def test_macro_steps_adaptive(oracle_mod, wname):
    w = small_c1() if wname == "c1" else small_c2()
    s, o = make_pair(w, oracle_mod)
    s.set_state(w.u0_cellmajor())
    u = np.ascontiguousarray(w.u0.copy())
    dtT_g = dtT_o = 15.0
    dtC_g = dtC_o = 0.5
    t = 0.0
    for step in range(3):
        rc, dtT_g, dtC_g, st = s.macro_step(t, t + 600.0, dtT_g, dtC_g)
        orc, dtT_o, dtC_o, ost = o.macro_step(u, t, t + 600.0, dtT_o, dtC_o)
        assert orc == 0
        assert (st.naT, st.nrT, st.naC, st.nrC) == tuple(ost[:4])
        assert dtT_g == pytest.approx(dtT_o, rel=1e-8)
        assert dtC_g == pytest.approx(dtC_o, rel=1e-8)
        t += 600.0
    ok, worst = close(s.get_state(), cm(w, u), rel=REL, floor=1e-9)
    assert ok, worst


@pytest.mark.parametrize("strict,precision", [(False, abi.RS_PREC_FP64), (True, abi.RS_PREC_FP64),
                                              (False, abi.RS_PREC_MIXED)])
def test_cwc_freestream_exact(strict, precision):
    """q == 1 with q_bc == 1 stays EXACTLY 1 under divergent open-wall flow
    (prototypes/transport_3d/transport_3d.esm freestream test; tools/cwc_gate.jl), in the
    FP64 builds and in the mixed-precision transport."""
    from reseact.esm_gb300 import mechanism
    g, mx, my, mz, dp = workloads.regional_freestream()
    mech = mechanism.superfast()
    n = g["nlon"]
    dp3 = np.broadcast_to(dp[:, None, None], (n, n, n)).copy()
    qb_lon = np.ones((mech.ns, n, n))
    f = abi.ForcingABI(mx=mx, my=my, mz=mz, dp=dp3, qbc_w=qb_lon, qbc_e=qb_lon, qbc_s=qb_lon,
                       qbc_n=qb_lon)
    mabi = abi.MechanismABI(mech)
    cfg = abi.make_config(g, mabi, do_chemistry=False, precision=precision)
    s = Solver(cfg, mabi, strict=strict)
    s.set_forcing(f)
    u = np.concatenate([np.ones((mech.ns, n, n, n)), dp3[None] * (1 + 0.1 * np.random.default_rng(0).random((1, n, n, n)))])
    s.set_state(workloads.soa_to_cellmajor(u, n, n, n))
    du = s.rhs_transport(workloads.soa_to_cellmajor(u, n, n, n)).reshape(-1, mech.ns + 1)
    assert np.all(du[:, :-1] == 0.0)
    dtT, dtC = 0.05, 1.0
    for k in range(4):
        rc, dtT, dtC, st = s.macro_step(0.1 * k, 0.1 * (k + 1), dtT, dtC)
    out = s.get_state().reshape(-1, mech.ns + 1)
    assert np.all(out[:, :-1] == 1.0)


def _c3_pair(oracle_mod, strict, ncells=2048, **kw):
    w = workloads.c3(ncells=ncells)
    mabi = abi.MechanismABI(w.mech)
    cfg = w.config(mabi, **kw)
    s = Solver(cfg, mabi, strict=strict)
    f = w.forcing_abi()
    s.set_forcing(f)
    o = oracle_mod.Oracle(cfg, f, mabi)
    o.set_lu_order(s.lu_order())
    o.set_rates(s.rates())
    s.set_state(w.u0_cellmajor())
    return w, cfg, s, o


@pytest.mark.parametrize("strict", [False, True])
def test_per_cell_single_attempt(oracle_mod, strict):
    """One attempt per cell of the persistent per-cell kernel (maxiters = 1) on the synthetic
    30-species / 60-reaction mechanism (the large kernel instantiation): strict build bit for
    bit, production build to roundoff."""
    w, cfg, s, o = _c3_pair(oracle_mod, strict, maxiters=1)
    u = np.ascontiguousarray(w.u0.copy())
    rc, _, _, st = s.macro_step(0.0, 600.0, 1.0, 0.05, check=False)
    assert rc == abi.RS_ERR_MAXITERS  # one attempt cannot reach t1
    orc, _, _ = o.chem_per_cell(u, 0.0, 600.0, 0.05)
    got, ref = s.get_state(), cm(w, u)
    if strict:
        assert np.array_equal(got, ref)
    else:
        err = np.abs(got - ref) / np.maximum(np.abs(ref), cfg.atol_C)
        assert err.max() < 1e-11, err.max()


@pytest.mark.parametrize("strict", [False, True])
def test_per_cell_mode_matches_oracle(oracle_mod, strict):
    """Per-cell adaptive chemistry (persistent work-queue kernel) against the oracle's per-cell
    loop over a whole 600 s window, uneven step counts, on the stiff synthetic mechanism
    (stiffness ratio ~1e8).  The solution of this problem is only determined to the
    integration tolerance: the oracle itself moves by up to ~1 x (rtol |u| + atol) when dt0
    changes by one ulp, and a cell whose accept/reject sequence flips on roundoff ends at a
    different valid point (checked by per_cell_agreement)."""
    w, cfg, s, o = _c3_pair(oracle_mod, strict)
    u = np.ascontiguousarray(w.u0.copy())
    rc, _, _, st = s.macro_step(0.0, 600.0, 1.0, 1e-3)
    orc, _, steps = o.chem_per_cell(u, 0.0, 600.0, 1e-3)
    assert rc == 0 and orc == 0
    assert steps.min() >= 1 and steps.max() > 2 * steps.min()  # uneven per-cell work
    per_cell_agreement(s.get_state(), cm(w, u), cfg, w.nsp)


def test_maxiters_is_reported_and_handle_stays_usable(oracle_mod):
    w = small_c2()
    s, _ = make_pair(w, oracle_mod, maxiters=2)
    s.set_state(w.u0_cellmajor())
    rc, _, _, st = s.macro_step(0.0, 600.0, 15.0, 0.5, check=False)
    assert rc == abi.RS_ERR_MAXITERS
    with pytest.raises(RsError):
        s.macro_step(0.0, 600.0, 15.0, 0.5)
    s.set_state(w.u0_cellmajor())  # still usable
    assert np.array_equal(s.get_state(), w.u0_cellmajor())


def test_nan_state_is_rejected_not_hung(oracle_mod):
    w = small_c2()
    s, _ = make_pair(w, oracle_mod, maxiters=50)
    u = w.u0_cellmajor().copy()
    u[5] = np.nan
    s.set_state(u)
    rc, _, _, st = s.macro_step(0.0, 600.0, 15.0, 0.5, check=False)
    assert rc in (abi.RS_ERR_MAXITERS, abi.RS_ERR_NONFINITE)


def test_bad_arguments():
    w = small_c2()
    s = Solver.for_workload(w)
    with pytest.raises(RsError):
        s.set_state(np.zeros(3))
    with pytest.raises(RsError):
        s.macro_step(10.0, 5.0, 1.0, 1.0)


def _tracer_masses(w, u_cm):
    g = w.grid
    u = workloads.cellmajor_to_soa(u_cm, w.nsp, g["nlon"], g["nlat"], g["nlev"])
    phie = workloads.lat_edges(g)
    area = (np.sin(np.radians(phie[1:])) - np.sin(np.radians(phie[:-1])))[None, :, None]
    m = u[-1]
    return np.array([(u[s] * m * area).sum() for s in range(w.nsp - 1)] + [(m * area).sum()])


def test_mixed_precision_transport_error_and_mass(oracle_mod):
    """FP32 reconstruction in deviation form with FP64 fluxes/divergence: agreement with the
    FP64 oracle to < 1e-6 relative after three transport-only macro steps, air mass conserved
    to roundoff and tracer-mass drift no worse than the FP64 scheme's own."""
    w = workloads.c2(nlon=36, nlat=19, nlev=10)
    s, o = make_pair(w, oracle_mod, do_chemistry=False, precision=abi.RS_PREC_MIXED)
    s.set_state(w.u0_cellmajor())
    u = np.ascontiguousarray(w.u0.copy())
    M0 = _tracer_masses(w, w.u0_cellmajor())
    t, dtT, dtTo = 0.0, 15.0, 15.0
    for _ in range(3):
        _, dtT, _, _ = s.macro_step(t, t + 600.0, dtT, 1.0)
        orc, dtTo, _, _ = o.macro_step(u, t, t + 600.0, dtTo, 1.0)
        t += 600.0
    got, ref = s.get_state(), cm(w, u)
    err = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-6)
    assert err.max() < 1e-6, err.max()
    Mg, Mo = _tracer_masses(w, got), _tracer_masses(w, ref)
    assert abs(Mg[-1] / M0[-1] - 1) < 1e-13
    drift_fp64 = np.abs(Mo[:-1] / M0[:-1] - 1)
    drift_mixed = np.abs(Mg[:-1] / M0[:-1] - 1)
    assert np.all(drift_mixed <= 10 * drift_fp64 + 1e-12)


def test_mixed_precision_full_step_within_1e6(oracle_mod):
    """The whole split step with mixed-precision transport (chemistry FP64) against the FP64
    oracle over three macro steps: max relative error < 1e-6 (atol floor)."""
    w = small_c2()
    s, o = make_pair(w, oracle_mod, precision=abi.RS_PREC_MIXED)
    s.set_state(w.u0_cellmajor())
    u = np.ascontiguousarray(w.u0.copy())
    t, a, b, ao, bo = 0.0, 15.0, 0.5, 15.0, 0.5
    for _ in range(3):
        _, a, b, _ = s.macro_step(t, t + 600.0, a, b)
        orc, ao, bo, _ = o.macro_step(u, t, t + 600.0, ao, bo)
        assert orc == 0
        t += 600.0
    got, ref = s.get_state(), cm(w, u)
    err = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-9)
    assert err.max() < 1e-6, err.max()


@pytest.mark.parametrize("strict", [False, True])
def test_minimum_grid_matches_oracle(oracle_mod, strict):
    """The smallest transport grid, 3 x 3 x 3 (every ghost position a wrapped or mirrored
    cell), through adaptive macro steps of transport and chemistry against the oracle, in
    both builds, with the same accept/reject counts."""
    w = workloads.c2(nlon=3, nlat=3, nlev=3, steps=1)
    mabi = abi.MechanismABI(w.mech)
    cfg = w.config(mabi)
    s = Solver(cfg, mabi, strict=strict)
    f = w.forcing_abi()
    s.set_forcing(f)
    o = oracle_mod.Oracle(cfg, f, mabi)
    o.set_lu_order(s.lu_order())
    o.set_rates(s.rates())
    s.set_state(w.u0_cellmajor())
    u = np.ascontiguousarray(w.u0.copy())
    t, a, b, ao, bo = 0.0, 15.0, 0.5, 15.0, 0.5
    for _ in range(2):
        _, a, b, st = s.macro_step(t, t + 600.0, a, b)
        _, ao, bo, ost = o.macro_step(u, t, t + 600.0, ao, bo)
        assert (st.naT, st.nrT, st.naC, st.nrC) == tuple(ost[:4])
        t += 600.0
    ok, worst = close(s.get_state(), workloads.soa_to_cellmajor(u, 3, 3, 3), rel=REL, floor=1e-9)
    assert ok, worst
