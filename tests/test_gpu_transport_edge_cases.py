"""Transport parity on the inputs where the production build's integer-pipe PPM forms could
differ from the FP forms: an identically zero species (signed zeros), piecewise-constant
plateaus (exact ties in every slope and limiter test) and fields of magnitude ~1e-199
(products of neighbour differences underflow, scalings stay normal).  Two transport-only
adaptive macro steps against the oracle: the strict build bit for bit, the production build
within 1e-10 relative (floor scaled to the field), the mixed-precision mode within 1e-6; a zero
species stays exactly zero in all three.
"""
import numpy as np
import pytest

from reseact.esm_gb300 import Solver, abi, workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def oracle_mod():
    from oracle import oracle
    oracle.build()
    return oracle


def _field(w, kind):
    g = w.grid
    u = np.array(w.u0, copy=True)
    ntr = w.nsp - 1
    k, j, i = np.meshgrid(np.arange(g["nlev"]), np.arange(g["nlat"]), np.arange(g["nlon"]),
                          indexing="ij")
    if kind == "zero":
        u[0] = 0.0
        u[4] = -0.0
    elif kind == "plateau":
        for s in range(ntr):
            u[s] = 1e-9 * (1.0 + ((i // 4 + j // 3 + k // 2 + s) % 3))
    elif kind == "tiny":
        u[:ntr] *= 1e-190
    return u


def _steps(solver_or_oracle, u, is_oracle, steps=2):
    t, dtT = 0.0, 15.0
    for _ in range(steps):
        if is_oracle:
            rc, dtT, _, _ = solver_or_oracle.macro_step(u, t, t + 600.0, dtT, 1.0)
        else:
            rc, dtT, _, _ = solver_or_oracle.macro_step(t, t + 600.0, dtT, 1.0)
        assert rc == 0
        t += 600.0


@pytest.mark.parametrize("kind", ["zero", "plateau", "tiny"])
@pytest.mark.parametrize("mode", ["strict", "production", "mixed"])
def test_transport_edge_fields_against_oracle(oracle_mod, kind, mode):
    w = workloads.c2(nlon=16, nlat=9, nlev=6, steps=1)
    g = w.grid
    mabi = abi.MechanismABI(w.mech)
    kw = dict(do_chemistry=False)
    if mode == "mixed":
        kw["precision"] = abi.RS_PREC_MIXED
    cfg = w.config(mabi, **kw)
    s = Solver(cfg, mabi, strict=(mode == "strict"))
    f = w.forcing_abi()
    s.set_forcing(f)
    o = oracle_mod.Oracle(w.config(mabi, do_chemistry=False), f, mabi)
    u = np.ascontiguousarray(_field(w, kind))
    s.set_state(workloads.soa_to_cellmajor(u, g["nlon"], g["nlat"], g["nlev"]))
    _steps(s, None, False)
    _steps(o, u, True)
    got = s.get_state()
    ref = workloads.soa_to_cellmajor(u, g["nlon"], g["nlat"], g["nlev"])
    s.close()
    nsp = w.nsp
    if kind == "zero":
        out = got.reshape(-1, nsp)
        assert np.all(out[:, 0] == 0.0) and np.all(out[:, 4] == 0.0)
    if mode == "strict":
        assert np.array_equal(got, ref)
        return
    if mode == "mixed" and kind == "tiny":
        # deviations below the FP32 range flush in the FP32 reconstruction: the faces fall back
        # to the upwind values (first order); the state stays finite and non-negative
        assert np.all(np.isfinite(got)) and np.all(got >= 0.0)
        return
    scale = np.abs(ref).reshape(-1, nsp).max(axis=0)
    floor = 1e-9 * np.tile(scale, ref.size // nsp)
    rel = np.abs(got - ref) / np.maximum(np.abs(ref), np.maximum(floor, 1e-300))
    tol = 1e-10 if mode == "production" else 1e-6
    assert rel.max() < tol, (kind, mode, rel.max())
