"""Algorithm 14 at the C ABI, on the CPU: option grammar, frozen rules, the
modeled property bytes and the learned model file.

The expected values are the reference's own (ParseDeployableSelectionPolicy,
ShouldUseAllKernelLowReuseRule, ShouldUseBudgetedLeidenGorder,
ModeledPropertyBytes; tests/golden/make_golden_selector.py).  The learned
model's model token is this library's addition.
"""
import ctypes as C
import json
import os

import numpy as np
import pytest

import graphbrew_gb300 as gb
from graphbrew_gb300 import selector as sel

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = json.load(open(os.path.join(HERE, "golden", "selector_cases.json")))


@pytest.mark.parametrize("case", CASES["policies"], ids=lambda c: c["opts"] or "<empty>")
def test_policy_grammar_matches_reference(case):
    if "error" in case:
        with pytest.raises(ValueError) as e:
            gb.parse_selection_policy(case["opts"])
        assert str(e.value) == case["error"]
    else:
        p = gb.parse_selection_policy(case["opts"])
        assert (p["model"], p["criterion"], p["reuse"], p["explicit"]) == \
            (case["model"], case["criterion"], case["reuse"], case["explicit"])


def test_learned_model_token():
    p = gb.parse_selection_policy("_:_:_:learned-mlp:best-endtoend:2")
    assert (p["model"], p["criterion"], p["reuse"], p["explicit"]) == (9, 2, 2.0, 1)
    assert gb.parse_selection_policy("_:_:_:mlp:e2e:1")["model"] == 9
    with pytest.raises(ValueError, match="learned-mlp requires an explicit reuse count"):
        gb.parse_selection_policy("_:_:_:learned-mlp:best-endtoend")
    assert gb.library().gbgpu_selection_model_name(9) == b"learned-mlp"
    assert gb.library().gbgpu_selection_criterion_name(2) == b"best-endtoend"


def test_frozen_rules_match_reference():
    lib = gb.library()
    for case in CASES["rules"]:
        n, avg, cv, hub, wsr = case["features"]
        f = (C.c_double * 9)(n, 0.0, avg, cv, 0.0, hub, 0.0, 0.0, 0.0)
        for model, key in ((8, "allkernel"), (7, "budgeted")):
            out = gb.GbgpuSelection()
            assert lib.gbgpu_apply_selection_rule(model, f, wsr, case["kernel"], case["reuse"], C.byref(out)) == 0
            assert (out.arm == 12) == bool(case[key]), (key, case)
            assert out.arm in (12, 5)


def test_property_bytes_match_reference():
    for case in CASES["property_bytes"]:
        assert gb.library().gbgpu_modeled_property_bytes(case["kernel"], case["nodes"], case["edges"]) == case["bytes"]


def test_python_rule_is_the_c_rule():
    """The Python selector's frozen rule (used for training and evaluation)
    decides as the C ABI's does on the same features."""
    rng = np.random.default_rng(3)
    lib = gb.library()
    for _ in range(500):
        t0 = np.array([rng.choice([800, 5000, 1e6]), 0, rng.uniform(1, 100), rng.uniform(0, 10), 0, 0, 0, 0, 0])
        kern = ["pr", "bfs", "cc"][rng.integers(3)]
        reuse = float(rng.choice([1, 2, 3]))
        cache = int(rng.choice([32 << 20, 126 << 20]))
        wsr = sel.working_set_ratio(t0, kern, cache)
        out = gb.GbgpuSelection()
        lib.gbgpu_apply_selection_rule(8, (C.c_double * 9)(*t0), wsr, gb.KERNELS[kern], reuse, C.byref(out))
        assert ("gb12" if out.arm == 12 else "dbg") == sel.frozen_rule(t0, kern, reuse, cache)


def test_model_file_round_trip(tmp_path):
    m = sel.LearnedSelector.load(os.path.join(os.path.dirname(gb.__file__), "data", "selector_mlp.npz"))
    path = str(tmp_path / "m.gbsel")
    m.save_binary(path)
    with open(path, "rb") as a, open(gb.SELECTOR_MODEL_PATH, "rb") as b:
        assert a.read() == b.read(), "committed model file is not the exported npz model"
    loaded = gb.SelectorModel(path)
    v = loaded.ptr.contents
    assert v.in_dim == len(m.mean) and v.cache_bytes == m.cache_bytes
    params = np.ctypeslib.as_array(C.cast(v.params, C.POINTER(C.c_float)), shape=(len(m.params),))
    np.testing.assert_array_equal(params, m.params)
    for name in ("mean", "std", "lo", "hi"):
        arr = np.ctypeslib.as_array(C.cast(getattr(v, name), C.POINTER(C.c_double)), shape=(v.in_dim,))
        np.testing.assert_array_equal(arr, getattr(m, name))
    loaded.close()
    bad = tmp_path / "bad.gbsel"
    bad.write_bytes(b"not a model")
    with pytest.raises(ValueError):
        gb.SelectorModel(str(bad))
