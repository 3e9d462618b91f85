"""The oracle equilibrium fixture (tests/golden/equilibrium_oracle.json) is the output of
make_equilibrium.py's case definitions: every case the GPU equilibrium tests use is present
with the generator's parameters, and a short fresh oracle run of one case agrees with it."""
import importlib.util
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = json.load(open(os.path.join(HERE, "golden", "equilibrium_oracle.json")))


def generator():
    spec = importlib.util.spec_from_file_location("make_equilibrium", os.path.join(HERE, "golden", "make_equilibrium.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_fixture_holds_every_case_with_its_parameters():
    gen = generator()
    assert set(gen.CASES) <= set(FIX)
    for name, case in gen.CASES.items():
        for k, v in case.items():
            assert FIX[name][k] == v, (name, k)
        for obs in ("E", "M") + (() if case["ising"] else ("Q",)):
            assert FIX[name][obs]["err"] > 0 and np.isfinite(FIX[name][obs]["mean"])


def test_short_oracle_run_agrees_with_the_fixture():
    gen = generator()
    case = dict(gen.CASES["ising_open_T23"])
    case.update(eq=500, samples=3000)
    res = [gen.run_chain((case, k)) for k in (100, 101)]
    assert res[0][0] == FIX["ising_open_T23"]["sites"]
    E = np.concatenate([r[1] for r in res])
    from stats import binned_error
    err = np.hypot(binned_error(E), FIX["ising_open_T23"]["E"]["err"])
    assert abs(E.mean() - FIX["ising_open_T23"]["E"]["mean"]) <= 5 * err
