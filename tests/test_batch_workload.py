"""The batched workload's specification (CPU): seeded, sizes in range."""
from graphbrew_gb300 import batch


def test_workload_seeded_and_in_range():
    a = batch.batch_workload(256, seed=1)
    b = batch.batch_workload(256, seed=1)
    assert a == b and len(a) == 256
    kinds = {k for k, _, _ in a}
    assert kinds == {"rmat", "planted"}
    for kind, n, p in a:
        if kind == "planted":
            assert 10_000 <= n <= 2_000_000 and 4 <= p["communities"] <= 64
        else:
            assert 2 ** 13 <= n <= 2 ** 21
