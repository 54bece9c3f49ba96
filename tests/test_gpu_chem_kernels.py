"""Mechanism-specialised chemistry kernels (straight-line CUDA generated from the mechanism
tables at rs_create and compiled for sm_103a with NVRTC) against the table-walking kernels
and the oracle, through the C ABI.  The strict build must give the same bits on both paths
(same arithmetic, same association); the production build agrees to roundoff."""
import numpy as np
import pytest

from reseact.esm_gb300 import Solver, abi, workloads
from reseact.esm_gb300._lib import CHEM_KERNEL_SPECIALIZED, CHEM_KERNEL_TABLE, RsError

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def oracle_mod():
    from oracle import oracle
    oracle.build()
    return oracle


def _small_c2(emission=False, seed=2, **kw):
    w = workloads.c2(seed=seed, nlon=16, nlat=9, nlev=6, steps=1)
    if emission:
        g = w.grid
        rng = np.random.default_rng(seed)
        e = np.zeros((w.mech.ns, g["nlev"], g["nlat"], g["nlon"]))
        e[w.mech.species.index("NO"), 0] = 1e-4 * np.exp(0.5 * rng.standard_normal((g["nlat"], g["nlon"])))
        w.forcing["emission"] = e
    return w


def _close(a, b, floor, rel=1e-12):
    err = np.abs(a - b) / np.maximum(np.abs(b), floor)
    return float(err.max())


def test_superfast_runs_specialised_kernels():
    s = Solver.for_workload(workloads.c1())
    kind, info = s.chem_kernel()
    assert kind == CHEM_KERNEL_SPECIALIZED, info
    assert info["kind"] == "specialized" and info["regs"][0] > 0


def test_large_mechanism_keeps_table_kernels():
    s = Solver.for_workload(workloads.c3(ncells=1024))
    kind, info = s.chem_kernel()
    assert kind == CHEM_KERNEL_TABLE and "why" in info
    with pytest.raises(RsError):
        s.set_chem_kernel(CHEM_KERNEL_SPECIALIZED)


@pytest.mark.parametrize("strict", [False, True])
@pytest.mark.parametrize("emission", [False, True])
def test_attempt_specialised_vs_table(strict, emission):
    w = _small_c2(emission)
    s = Solver.for_workload(w, strict=strict)
    u = w.u0_cellmajor()
    s.set_chem_kernel(CHEM_KERNEL_TABLE)
    a, ea = s.single_step(abi.RS_OP_CHEMISTRY, u, 0.0, 30.0)
    s.set_chem_kernel(CHEM_KERNEL_SPECIALIZED)
    b, eb = s.single_step(abi.RS_OP_CHEMISTRY, u, 0.0, 30.0)
    if strict:
        assert np.array_equal(a, b) and ea == eb
    else:
        assert _close(b, a, 1e-9) < 1e-12
        assert eb == pytest.approx(ea, rel=1e-11)


@pytest.mark.parametrize("strict", [False, True])
def test_attempt_specialised_vs_oracle(oracle_mod, strict):
    w = _small_c2(emission=True)
    mabi = abi.MechanismABI(w.mech)
    cfg = w.config(mabi)
    s = Solver(cfg, mabi, strict=strict)
    f = w.forcing_abi()
    s.set_forcing(f)
    assert s.chem_kernel()[0] == CHEM_KERNEL_SPECIALIZED
    o = oracle_mod.Oracle(cfg, f, mabi)
    o.set_lu_order(s.lu_order())
    o.set_rates(s.rates())
    un_o, e_o = o.single_step(abi.RS_OP_CHEMISTRY, w.u0, 0.0, 30.0)
    un_g, e_g = s.single_step(abi.RS_OP_CHEMISTRY, w.u0_cellmajor(), 0.0, 30.0)
    g = w.grid
    ref = workloads.soa_to_cellmajor(un_o, g["nlon"], g["nlat"], g["nlev"])
    if strict:
        assert np.array_equal(un_g, ref) and e_g == e_o
    else:
        assert _close(un_g, ref, 1e-9) < 1e-12
        assert e_g == pytest.approx(e_o, rel=1e-10)


@pytest.mark.parametrize("strict", [False, True])
def test_macro_steps_specialised_vs_table(strict):
    """Three adaptive macro steps (graph loop): identical accept/reject sequence; the strict
    build identical bits."""
    w = _small_c2(emission=True)
    out = []
    for kind in (CHEM_KERNEL_TABLE, CHEM_KERNEL_SPECIALIZED):
        s = Solver.for_workload(w, strict=strict)
        s.set_chem_kernel(kind)
        s.set_state(w.u0_cellmajor())
        t, a, b, counts = 0.0, 15.0, 0.5, []
        for _ in range(3):
            _, a, b, st = s.macro_step(t, t + 600.0, a, b)
            counts.append((st.naC, st.nrC))
            t += 600.0
        out.append((s.get_state(), counts, b))
        s.close()
    (ua, ca, ba), (ub, cb, bb) = out
    assert ca == cb
    if strict:
        assert np.array_equal(ua, ub) and ba == bb
    else:
        assert _close(ub, ua, 1e-9) < 1e-10


@pytest.mark.parametrize("strict", [False, True])
def test_per_cell_specialised_vs_table(strict):
    w = _small_c2(emission=True)
    out = []
    for kind in (CHEM_KERNEL_TABLE, CHEM_KERNEL_SPECIALIZED):
        s = Solver.for_workload(w, strict=strict, do_transport=False,
                                chem_mode=abi.RS_CHEM_PER_CELL)
        s.set_chem_kernel(kind)
        s.set_state(w.u0_cellmajor())
        _, _, _, st = s.macro_step(0.0, 600.0, 1.0, 0.5)
        out.append((s.get_state(), st.chem_cell_steps))
        s.close()
    (ua, na), (ub, nb) = out
    if strict:
        assert np.array_equal(ua, ub) and na == nb
    else:
        assert _close(ub, ua, 1e-9) < 1e-9


def test_autotuned_chemistry_variant_is_bitwise_neutral():
    w = _small_c2(emission=True)
    res = []
    for tune in (False, True):
        s = Solver.for_workload(w)
        s.set_state(w.u0_cellmajor())
        rep = s.autotune() if tune else None
        if tune:
            assert rep["chem_choice"] in ("regs", "smem", "regs2", "split")
            assert len(rep["chem_attempt"]) == 4
        t, a, b = 0.0, 15.0, 0.5
        for _ in range(2):
            _, a, b, _ = s.macro_step(t, t + 600.0, a, b)
            t += 600.0
        res.append(s.get_state())
        s.close()
    assert np.array_equal(res[0], res[1])


@pytest.mark.parametrize("strict", [False, True])
def test_every_attempt_variant_gives_the_same_bits(strict):
    """W in registers, in shared memory, capped at 128 registers, or split between shared
    memory and registers: the same generated arithmetic, so the same bits after adaptive
    macro steps."""
    w = _small_c2(emission=True)
    res = []
    for v in range(4):
        s = Solver.for_workload(w, strict=strict)
        s.set_launch_shape(chem_attempt_variant=v)
        s.set_state(w.u0_cellmajor())
        t, a, b = 0.0, 15.0, 0.5
        for _ in range(2):
            _, a, b, _ = s.macro_step(t, t + 600.0, a, b)
            t += 600.0
        res.append(s.get_state())
        s.close()
    for r in res[1:]:
        assert np.array_equal(res[0], r)


def test_production_reciprocal_within_two_ulp():
    """The refined hardware reciprocal (third-order correction r (1 + e + e^2)) that replaces
    IEEE division in the production build's specialised kernels, against the correctly rounded
    1/x, over the magnitudes the kernels divide by (LU pivots near 1, error-norm denominators
    from atol upwards)."""
    rng = np.random.default_rng(7)
    x = np.concatenate([10.0 ** rng.uniform(-30, 30, 200000), 1.0 + rng.uniform(0, 1e3, 50000),
                        np.array([1.0, 2.0, 3.0, 1e-9, 1.0 + 2.0 ** -52, 1.5, 7.0])])
    s = Solver.for_workload(workloads.c1())
    r = s.chem_kernel_reciprocal(x)
    ref = 1.0 / x
    ulp = np.abs(r - ref) / np.spacing(ref)
    assert ulp.max() <= 1.0, ulp.max()
    assert np.mean(r == ref) > 0.9  # mostly the correctly rounded value


@pytest.mark.parametrize("strict", [False, True])
def test_adjoint_specialised_vs_table(strict):
    """The specialised ROS23 step VJP (forward recompute, W^T solves, J^T products, the exact
    mass-action Hessian) against the table kernel over a recorded sweep: the strict build
    identical bits, the production build to roundoff."""
    w = _small_c2(emission=True)
    g = w.grid
    out = []
    for kind in (CHEM_KERNEL_TABLE, CHEM_KERNEL_SPECIALIZED):
        s = Solver.for_workload(w, strict=strict, do_transport=False)
        s.set_chem_kernel(kind)
        s.set_state(w.u0_cellmajor())
        s.record(True)
        t, a, b = 0.0, 15.0, 0.5
        for _ in range(2):
            _, a, b, _ = s.macro_step(t, t + 600.0, a, b)
            t += 600.0
        s.record(False)
        lam = np.zeros(s.n)
        lam[w.mech.species.index("O3")::w.nsp] = 1.0
        out.append(s.adjoint_backward(lam))
        s.close()
    (la, ea), (lb, eb) = out
    if strict:
        assert np.array_equal(la, lb) and np.array_equal(ea, eb)
    else:
        assert np.abs(lb - la).max() <= 1e-10 * np.abs(la).max()
        assert np.abs(eb - ea).max() <= 1e-10 * np.abs(ea).max()
