"""Algorithm 14 through the C ABI on the GPU: gbgpu_select_arm picks the arm
the Python selector (LearnedSelector.choose, frozen_rule) picks, on held-out
graphs of the training distribution, and gbconvert runs the chosen arm
through the builder lifecycle."""
import os
import subprocess

import numpy as np
import pytest
import torch

import graphbrew_gb300 as gb
from graphbrew_gb300 import graphgen as gg
from graphbrew_gb300 import selector as sel

pytestmark = pytest.mark.gpu
ARM_NAME = {12: "gb12", 5: "dbg", 0: "original"}
DATA = os.path.join(os.path.dirname(gb.__file__), "data")


@pytest.fixture(scope="module")
def ctx():
    c = gb.Context(0)
    yield c
    c.close()


def test_select_arm_matches_python_selector(ctx):
    model = gb.SelectorModel()
    learned = sel.LearnedSelector.load(os.path.join(DATA, "selector_mlp.npz"))
    l2 = torch.cuda.get_device_properties(0).L2_cache_size
    seen_arms, seen_how = set(), set()
    for seed in range(2000, 2016):
        _, _, rp, col = sel.random_graph(seed, scale_range=(12, 16))
        t0 = ctx.tier0_features(rp, col)
        for kern in ("pr", "bfs", "cc"):
            for reuse in (1, 2):
                d = ctx.select_arm(rp, col, f"_:_:_:learned-mlp:best-endtoend:{reuse}", kern, model)
                arm, how = learned.choose(ctx, t0, kern, reuse)
                assert (ARM_NAME[d["arm"]], d["reason"]) == (arm, how), (seed, kern, reuse, d)
                np.testing.assert_array_equal(np.array(d["features"]), t0)
                seen_arms.add(arm)
                seen_how.add(how)
                f = ctx.select_arm(rp, col, f"_:_:_:allkernel-lowreuse-rule:best-endtoend:{reuse}", kern)
                assert ARM_NAME[f["arm"]] == sel.frozen_rule(t0, kern, reuse, l2)
                assert f["cache_bytes"] == l2
                assert f["reason"] in ("allkernel-lowreuse-match", "allkernel-lowreuse-fallback")
    assert len(seen_arms) >= 2, seen_arms
    model.close()


def test_select_arm_errors(ctx):
    rp, col = gg.gapbs(10, 16, device="cuda")
    with pytest.raises(ValueError, match="Kernel-specific modeled property bytes are unavailable"):
        ctx.select_arm(rp, col, "_:_:_:allkernel-lowreuse-rule:best-endtoend:1", "generic")
    with pytest.raises(ValueError, match="requires best-endtoend criterion"):
        ctx.select_arm(rp, col, "_:_:_:allkernel-lowreuse-rule:execution:1", "pr")
    with pytest.raises(NotImplementedError):
        ctx.select_arm(rp, col, "_:_:_:perceptron:best-endtoend", "pr")
    with pytest.raises(ValueError, match="needs a model"):
        ctx.select_arm(rp, col, "_:_:_:learned-mlp:best-endtoend:1", "pr")


@pytest.mark.parametrize("model_tok", ["allkernel-lowreuse-rule", "learned-mlp"])
def test_cli_algorithm_14(model_tok):
    cli = os.path.join(os.path.dirname(gb.__file__), "gbconvert")
    r = subprocess.run([cli, "-g", "14", "-s", "-K", "pr", "-o", f"14:_:_:_:{model_tok}:best-endtoend:1"],
                       check=True, capture_output=True, text=True)
    out = r.stdout
    assert "=== Full-Graph Adaptive Mode (Standalone) ===" in out
    assert f"Selection: model={model_tok} criterion=best-endtoend" in out
    applied = next(l for l in out.splitlines() if l.startswith("Adaptive Applied:")).split(":", 1)[1].strip()
    assert applied in ("5", "0") or applied.startswith("12:leiden:compose")
    for label in ("Mapping Fingerprint", "Reorder End-to-End Time", "Adaptive Override Reason"):
        assert label + ":" in out
    bad = subprocess.run([cli, "-g", "10", "-s", "-o", "14:_:_:_:allkernel-lowreuse-rule:best-endtoend:1"],
                         capture_output=True, text=True)
    assert bad.returncode == 2 and "Kernel-specific modeled property bytes are unavailable" in bad.stderr
