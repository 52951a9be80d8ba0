"""Option grammar and the C ABI surface (CPU only: no compute calls).

The effective-config JSON of every option string must be byte-identical to the
reference's (graphBrewEffectiveConfigJson, reorder_graphbrew.h:693-775), and
rejected strings must carry the reference's exception text.
"""
import ctypes
import os
import re

import pytest

import graphbrew_gb300 as gb
from conftest import ROOT


def test_library_exports_every_declared_symbol():
    header = open(os.path.join(ROOT, "include", "gbgpu.h")).read()
    declared = set(re.findall(r"\b(gbgpu_[a-z_0-9]+)\s*\(", header))
    assert declared, "no declarations found"
    lib = ctypes.CDLL(gb.LIB_PATH)
    missing = [s for s in sorted(declared) if not hasattr(lib, s)]
    assert not missing, missing
    assert declared == set(gb.SIGNATURES), declared ^ set(gb.SIGNATURES)


def test_parser_matches_reference_corpus(parser_cases):
    mismatches = []
    for case in parser_cases:
        try:
            _, text = gb.parse_graphbrew_config(case["options"], case["auto_resolution"])
            ok = True
        except (ValueError, NotImplementedError) as e:
            text, ok = str(e), False
        if ok != case["ok"] or text != case["text"]:
            mismatches.append((case["options"], case["ok"], ok, case["text"][:120], text[:120]))
    assert not mismatches, mismatches[:5]


def test_recipe_fields():
    cfg, _ = gb.parse_graphbrew_config(gb.DEFAULT_RECIPE, 0.5)
    # bench/tests/test_graphbrew_config.cc:309-317 asserts these for the recipe.
    assert cfg["super_move_batch"] == 4096
    assert cfg["gorder_fallback"] == 5000
    assert cfg["use_refinement"] == 0
    assert cfg["max_iterations"] == 2 and cfg["max_passes"] == 2
    assert cfg["gorder_window"] == 8
    assert cfg["deterministic"] == 0
    assert cfg["resolution"] == 0.5


def test_preset_tail_parsing():
    # bench/tests/test_graphbrew_config.cc:145-183
    eff = gb.effective_config("leiden:compose:sg_super_rabbit:comm_identity:intra_gorder:gw8", 0.75)
    assert eff["aggregation"] == "gve-csr"
    assert eff["m_computation"] == "total-edges"
    assert eff["ordering"] == "compose"
    assert eff["super_graph"] == "super-rabbit"
    assert eff["community_order"] == "identity"
    assert eff["intra_community_order"] == "gorder"
    assert eff["gorder_window"] == 8


def test_fail_closed_tokens():
    with pytest.raises(ValueError, match="Unknown or invalid GraphBrew option: sgmb0"):
        gb.parse_graphbrew_config("leiden:compose:sgmb0")
    with pytest.raises(ValueError, match="positional integer is malformed"):
        gb.parse_graphbrew_config("leiden:1.5")


def test_fingerprint_abi_matches_builder_definition():
    import numpy as np
    ids = np.array([3, 1, 0, 2], dtype=np.int32)
    h = 1469598103934665603
    for i, v in enumerate(ids):
        h ^= i
        h = (h * 1099511628211) & (2**64 - 1)
        h ^= int(v)
        h = (h * 1099511628211) & (2**64 - 1)
    assert gb.mapping_fingerprint(ids) == "%016x" % h
