"""Batched mode (GB300): concurrent worker streams give every graph exactly
the single-call permutation, for every schedule."""
import numpy as np
import pytest
import torch

import graphbrew_gb300 as gb
from graphbrew_gb300 import batch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    c = gb.Context(0)
    yield c
    c.close()


def test_batched_equals_single(ctx):
    specs = batch.batch_workload(8, seed=5, n_min=2e3, n_max=6e4)
    graphs = [batch.make_graph(s) for s in specs]
    single = [ctx.generate_mapping(rp, col)[0] for rp, col in graphs]
    for sched in ({"streams": 3, "order": 1, "exact_window": 0}, {"streams": 1, "order": 0, "exact_window": 4096}):
        ids, stats, wall = ctx.generate_mappings_batched(graphs, **sched)
        assert wall > 0 and len(stats) == len(graphs)
        for a, b, (rp, _) in zip(ids, single, graphs):
            np.testing.assert_array_equal(a.cpu().numpy(), b.cpu().numpy())
            assert ctx.validate_permutation(a) == 0


def test_autotune_small(ctx):
    specs = batch.batch_workload(6, seed=9, n_min=2e3, n_max=3e4)
    graphs = [batch.make_graph(s) for s in specs]
    cands = [{"streams": s, "order": 1, "exact_window": 0} for s in (1, 2)]
    best, table = batch.autotune(ctx, graphs, sample=6, candidates=cands)
    assert best in cands and len(table) == 2
