"""Pin the algorithm-14 selection pieces against the GraphBrew reference.

Run where the GraphBrew sources are mounted and the reference harness is built
(``make -C oracle ref``):

    python tests/golden/make_golden_selector.py

It records, through oracle/ref_harness.cc,
  * ParseDeployableSelectionPolicy (reorder_adaptive.h:166-228) on option
    strings after "14:": model / criterion ordinals, reuse, whether the reuse
    was given -- or the exception text;
  * ShouldUseAllKernelLowReuseRule and ShouldUseBudgetedLeidenGorder
    (reorder_adaptive.h:240-333) on seeded feature vectors around their
    thresholds, for every benchmark kind and several reuse counts;
  * ModeledPropertyBytes (reorder_types.h:1226-1258) for every kind.
Output: ``selector_cases.json``.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import random
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import pyoracle as po  # noqa: E402

POLICIES = [
    "", "_:_:_", "_:_:_:allkernel-lowreuse-rule:best-endtoend:1", "_:_:_:allkernel-lowreuse-rule:best-endtoend:2",
    "_:_:_:allkernel-lowreuse-rule:best-endtoend", "_:_:_:allkernel-rule:e2e:1.5", "_:_:_:lowreuse-rule:endtoend:0.5",
    "_:_:_:allkernel-lowreuse-rule:execution:1", "_:_:_:budgeted-rule:best-endtoend:1", "_:_:_:budgeted:e2e:1",
    "_:_:_:one-use-rule:e2e", "_:_:_:perceptron:best-endtoend", "_:_:_:perceptron", "_:_:_:p:fe",
    "_:_:_:perceptron:best-amortization:3", "_:_:_:knn:execution", "_:_:_:decision-tree:execution",
    "_:_:_:dt", "_:_:_:4", "_:_:_:0", "_:_:_:1", "_:_:_:2", "_:_:_:3", "_:_:_:e2e", "_:_:_:hybrid",
    "_:_:_:perceptron:twitter7", "_:_:_:unknown-model", "garbage", "_:x:_", "_:_:y:perceptron",
    "_:_:_:perceptron:execution:twitter7", "_:_:_:perceptron:execution:1:_", "_:_:_:perceptron:execution:1:x",
    "_:_:_:_:best-endtoend:1", "_:_:_:_:_:2", "_:_:_:allkernel-lowreuse-rule:best-endtoend:0",
    "_:_:_:allkernel-lowreuse-rule:best-endtoend:-1", "_:_:_:allkernel-lowreuse-rule:best-endtoend:abc",
    "_:_:_:allkernel-lowreuse-rule:best-endtoend:1x", "_:_:_:allkernel-lowreuse-rule:best-endtoend:nan",
    "_:_:_:allkernel-lowreuse-rule:best-endtoend:inf", "_:_:_:allkernel-lowreuse-rule:best-endtoend:1e3",
    "_:_:_:family", "_:_:_:topn:execution", "_:_:_:individual", "_:_:_:perc:reorder:2",
    "_:_:_:budgeted-rule", "_:_:_:fastest-reorder", "_:_:_:cache", "_:_:_:amortize", "_:_:_:db",
    "::", ":::allkernel-lowreuse-rule:best-endtoend:1", ":::perceptron:e2e:",
]


def main():
    ref = po.load_reference()
    if ref is None:
        sys.exit("reference harness not built (make -C oracle ref)")
    ref.ref_parse_selection_policy.argtypes = [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                               C.POINTER(C.c_double), C.POINTER(C.c_int), C.c_char_p, C.c_size_t]
    ref.ref_allkernel_rule.argtypes = [C.c_double] * 5 + [C.c_int, C.c_double]
    ref.ref_budgeted_rule.argtypes = [C.c_double] * 4 + [C.c_int, C.c_double]
    ref.ref_property_bytes.restype = C.c_longlong
    ref.ref_property_bytes.argtypes = [C.c_int, C.c_ulonglong, C.c_ulonglong]
    out = {"policies": [], "rules": [], "property_bytes": []}
    for opts in POLICIES:
        m, c, x = C.c_int(), C.c_int(), C.c_int()
        r = C.c_double()
        err = C.create_string_buffer(512)
        rc = ref.ref_parse_selection_policy(opts.encode(), C.byref(m), C.byref(c), C.byref(r), C.byref(x), err, 512)
        rec = {"opts": opts}
        if rc == 0:
            rec.update({"model": m.value, "criterion": c.value, "reuse": r.value, "explicit": x.value})
        else:
            rec["error"] = err.value.decode()
        out["policies"].append(rec)
    rnd = random.Random(14)
    for _ in range(3000):
        f = [float(rnd.choice([500, 999, 1000, 1001, 5000, 10 ** 6])), rnd.uniform(1, 120), rnd.uniform(0, 12),
             rnd.uniform(0, 1), rnd.uniform(0, 5)]
        # thresholds exactly, too
        if rnd.random() < 0.2:
            f[1] = rnd.choice([45.0, 60.0, 60.000001])
        if rnd.random() < 0.2:
            f[2] = rnd.choice([2.68, 3.0, 8.0, 8.000001])
        if rnd.random() < 0.2:
            f[4] = rnd.choice([0.82, 3.2, 3.2000001])
        if rnd.random() < 0.1:
            f[3] = 0.3
        kernel = rnd.randrange(9)
        reuse = rnd.choice([0.5, 1.0, 1.5, 2.0, 2.5, 3.0])
        out["rules"].append({"features": f, "kernel": kernel, "reuse": reuse,
                             "allkernel": ref.ref_allkernel_rule(*f, kernel, reuse),
                             "budgeted": ref.ref_budgeted_rule(*f[:4], kernel, reuse)})
    for kernel in range(9):
        for nodes, edges in ((0, 0), (1, 0), (7, 12), (1000, 16000), (4194302, 128311450), (1 << 30, 1 << 34)):
            out["property_bytes"].append({"kernel": kernel, "nodes": nodes, "edges": edges,
                                          "bytes": ref.ref_property_bytes(kernel, nodes, edges)})
    with open(os.path.join(HERE, "selector_cases.json"), "w") as fh:
        json.dump(out, fh, indent=0)
        fh.write("\n")
    print(len(out["policies"]), "policies", sum(1 for p in out["policies"] if "error" in p), "rejected")


if __name__ == "__main__":
    main()
