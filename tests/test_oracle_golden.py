"""Pin the CPU oracle to the reference's own golden vectors.

The SuperFast reaction system carries six inline tests with 49 assertions
(prototypes/g2_depsink/g2_nodep.esm:9-400; "reference run from upstream GasChem.jl
Rosenbrock23").  The oracle integrates each 0-D box with its ROS23 + PI controller at tight
tolerance and must land inside every assertion's tolerance.  The same run decides the
mass-action convention: plain k*prod(x^nu) passes, the combinatoric k*prod(x^nu)/nu! fails.
"""
import numpy as np
import pytest

from reseact.esm_gb300 import abi, mechanism


def run_box_test(oracle, mech, test, tol=1e-10):
    m = mech.with_params(**test.get("parameter_overrides", {}))
    mabi, cfg = oracle.box_model(m, tol=tol, atol=1e-20)
    f = abi.ForcingABI(temperature=np.full((1, 1, 1), 280.0),
                       pressure=np.full((1, 1, 1), 101325.0), dp=np.ones((1, 1, 1)))
    o = oracle.Oracle(cfg, f, mabi)
    u = np.array([m.defaults[s] for s in m.species]).reshape(m.ns, 1, 1, 1)
    for k, v in test.get("initial_conditions", {}).items():
        u[m.species.index(k)] = v
    t = float(test["time_span"]["start"])
    dtC = 1e-3
    out = []
    for ts in sorted({a["time"] for a in test["assertions"]}):
        if ts > t:
            rc, _, dtC, _ = o.macro_step(u, t, float(ts), 1.0, dtC)
            assert rc == 0
            t = float(ts)
        for a in test["assertions"]:
            if a["time"] != ts:
                continue
            tl = dict(test.get("tolerance", {}))
            tl.update(a.get("tolerance", {}))
            got = float(u[m.species.index(a["variable"])].item())
            err = abs(got - a["expected"])
            bound = max(tl.get("rel", 1e-4) * abs(a["expected"]), tl.get("abs", 0.0))
            out.append((test["id"], a["variable"], ts, a["expected"], got, err, bound))
    return out


@pytest.fixture(scope="module")
def results(oracle_lib):
    res = {}
    for comb in (False, True):
        mech = mechanism.superfast(combinatoric=comb)
        rows = []
        for test in mech.tests:
            rows += run_box_test(oracle_lib, mech, test)
        res[comb] = rows
    return res


def test_superfast_golden_all_assertions(results):
    rows = results[False]
    assert len(rows) == 49
    bad = [r for r in rows if not r[5] <= r[6]]
    assert not bad, bad


def test_combinatoric_convention_is_rejected(results):
    bad = [r for r in results[True] if not r[5] <= r[6]]
    assert len(bad) > 10


def test_initial_conditions_exact(oracle_lib):
    mech = mechanism.superfast()
    t0 = [t for t in mech.tests if t["id"] == "initial_conditions_t0"][0]
    for a in t0["assertions"]:
        assert mech.defaults[a["variable"]] == pytest.approx(a["expected"], rel=1e-10, abs=1e-14)
