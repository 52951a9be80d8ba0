"""Learned selector against the frozen rule (GB300).

The committed dataset (``graphbrew_gb300/data/selector_records.npz``) holds
GPU-measured map + PR/BFS/CC times of the three arms on 2,000 training and
200 held-out seeded graphs (``python -m graphbrew_gb300.selector collect``).
Training on the GPU is deterministic for a fixed seed, so the held-out
comparison is reproducible: the learned choices' total end-to-end time must
not exceed the frozen rule's.
"""
import os

import numpy as np
import pytest
import torch

import graphbrew_gb300 as gb
from graphbrew_gb300 import selector as sel

pytestmark = pytest.mark.gpu

DATA = os.path.join(os.path.dirname(sel.__file__), "data", "selector_records.npz")


@pytest.fixture(scope="module")
def ctx():
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    c = gb.Context(0)
    yield c
    c.close()


def test_measure_graph_small(ctx):
    """One live measurement: every arm and kernel timed, features finite."""
    fam, scale, rp, col = sel.random_graph(3, scale_range=(14, 14))
    tier0, map_ms, kms = sel.measure_graph(ctx, rp, col, repeats=1)
    assert np.isfinite(tier0).all() and tier0[0] == rp.numel() - 1
    assert map_ms[0] > 0 and map_ms[1] > 0 and map_ms[2] == 0
    assert (kms > 0).all()


@pytest.mark.skipif(not os.path.exists(DATA), reason="selector dataset not collected")
def test_learned_selector_beats_frozen_rule_on_heldout(ctx):
    data = dict(np.load(DATA))
    cache = int(data.get("l2_bytes", sel.GB300_L2_BYTES))
    train, held = sel.split_masks(data)
    assert train.sum() >= 1000 and held.sum() >= 100
    X, T, _ = sel.dataset_rows(data, train, cache)
    model = sel.LearnedSelector.train(ctx, X, T, epochs=300, cache_bytes=cache)
    res = sel.evaluate(ctx, model, data, held)
    assert res["rows"] == held.sum() * 6
    # What the network gains over the rule on graphs it never saw.
    assert res["learned_ms"] <= res["frozen_ms"], res
    assert res["learned_ms"] >= res["best_ms"]
