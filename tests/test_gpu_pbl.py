"""Full PBL mixing on the GPU (the first of the next rows: a transport-half column term,
reseact.esm Transport3D pbl_f*(pbl_mean - q)/tau_pblmix) against the oracle through the C ABI:
the transport RHS bit for bit in the strict build, adaptive macro steps to 1e-10, column mass
conservation, and the discrete adjoint with the term's VJP."""
import numpy as np
import pytest

from reseact.esm_gb300 import Solver, abi, workloads

pytestmark = pytest.mark.gpu

REL = 1e-10


@pytest.fixture(scope="module")
def oracle_mod():
    from oracle import oracle
    oracle.build()
    return oracle


def _w(still=False, **kw):
    w = workloads.c2(nlon=16, nlat=9, nlev=12, steps=1)
    if still:
        for k in ("mx", "my", "mz"):
            w.forcing[k] = np.zeros_like(w.forcing[k])
    return workloads.with_pbl(w, pblh_median=2500.0, **kw)


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
def test_transport_rhs_with_pbl(oracle_mod, strict):
    w = _w(tau=300.0)
    s, o = _pair(w, oracle_mod, strict=strict)
    base = workloads.c2(nlon=16, nlat=9, nlev=12, steps=1)
    s0, _ = _pair(base, oracle_mod, strict=strict)
    for t in (0.0, 3600.0):
        du_o = cm(w, o.rhs_transport(w.u0, t))
        du_g = s.rhs_transport(w.u0_cellmajor(), t)
        assert not np.array_equal(du_g, s0.rhs_transport(w.u0_cellmajor(), t))  # the term acts
        if strict:
            assert np.array_equal(du_g, du_o)
        else:
            scale = np.abs(du_o).reshape(-1, w.nsp).max(axis=0)
            err = np.abs(du_g - du_o).reshape(-1, w.nsp) / scale
            assert err.max() < 1e-12, err.max()


@pytest.mark.parametrize("precision", [abi.RS_PREC_FP64, abi.RS_PREC_MIXED])
def test_macro_steps_with_pbl(oracle_mod, precision):
    """FP64 and the compensated FP32 transport (whose stage kernel forms the tendency with the
    PBL term in FP64 from the pair accumulator) against the FP64 oracle."""
    w = _w(tau=900.0)
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
    assert err.max() < REL, err.max()


def test_pbl_conserves_column_mass_on_gpu():
    w = _w(still=True, tau=120.0)
    s = Solver.for_workload(w, do_chemistry=False)
    s.set_state(w.u0_cellmajor())
    dp = np.asarray(w.forcing["dp"])
    ntr = w.mech.ns
    m0 = (w.u0[:ntr] * dp[None]).sum(axis=1)
    s.macro_step(0.0, 1800.0, 15.0, 0.5)
    g = w.grid
    u = workloads.cellmajor_to_soa(s.get_state(), w.nsp, g["nlon"], g["nlat"], g["nlev"])
    m1 = (u[:ntr] * dp[None]).sum(axis=1)
    assert np.abs(m1 / m0 - 1).max() < 1e-12
    assert not np.allclose(u[:ntr], w.u0[:ntr], rtol=1e-6)  # the profiles did mix


def test_adjoint_with_pbl_matches_oracle(oracle_mod):
    w = _w(tau=600.0)
    g = w.grid
    s, o = _pair(w, oracle_mod)
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
    iO3 = w.mech.species.index("O3")
    uend = workloads.cellmajor_to_soa(s.get_state(), w.nsp, g["nlon"], g["nlat"], g["nlev"])
    lam = np.zeros_like(uend)
    lam[iO3, 0] = 2 * uend[iO3, 0]
    lg, _ = s.adjoint_backward(workloads.soa_to_cellmajor(lam, g["nlon"], g["nlat"], g["nlev"]))
    lo, _ = o.adjoint_backward(lam)
    lo = cm(w, lo)
    scale = np.abs(lo).max()
    assert np.abs(lg - lo).max() <= 1e-8 * scale, np.abs(lg - lo).max() / scale
    # the PBL term couples the column: the surface objective reaches layers above level 0
    lg3 = workloads.cellmajor_to_soa(lg, w.nsp, g["nlon"], g["nlat"], g["nlev"])
    assert np.abs(lg3[iO3, 1:4]).max() > 1e-6 * np.abs(lg3[iO3, 0]).max()
