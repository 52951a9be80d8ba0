"""The allocation-free permutation check, through the C ABI.

gbgpu_validate_permutation_noalloc exists for callers that cannot allocate
device memory (a process whose GPU memory belongs to another framework's
allocator, latency-critical loops that cannot take cudaMalloc's implicit
synchronisation).  It must give the same
answers as gbgpu_validate_permutation, call after call, although every call
reuses one fixed scratch array that still holds the previous call's data.

This file is collected last so that a run stopping at its first failure has
already run every other test; it also passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest
import torch

import graphbrew_gb300 as gb

pytestmark = pytest.mark.gpu

MAX_N = 1 << 20  # GBGPU_NOALLOC_MAX_VERTICES


def _noalloc(ctx, ids_dev):
    res = ctypes.c_int32(-1)
    rc = gb.library().gbgpu_validate_permutation_noalloc(ctx.handle, ctypes.c_void_p(ids_dev.data_ptr()),
                                                         ids_dev.numel(), ctypes.byref(res))
    return rc, res.value


def _reference_answer(ctx, ids_dev):
    res = ctypes.c_int32(-1)
    rc = gb.library().gbgpu_validate_permutation(ctx.handle, ctypes.c_void_p(ids_dev.data_ptr()), ids_dev.numel(),
                                                 gb.DEVICE_POINTERS, ctypes.byref(res))
    assert rc == gb.OK
    return res.value


def test_noalloc_matches_allocating_check_call_after_call():
    assert torch.cuda.is_available()
    ctx = gb.Context(0)
    rng = np.random.default_rng(7)
    valid = torch.from_numpy(rng.permutation(MAX_N).astype(np.int32)).cuda()
    dup = valid.clone()
    dup[123456] = dup[42]
    small_oor = torch.tensor([3, 0, 7, 1], dtype=torch.int32, device="cuda")
    small_valid = torch.tensor([3, 0, 2, 1], dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()

    # First call sets the scratch address up for this device.
    rc, r = _noalloc(ctx, valid)
    assert rc == gb.OK and r == _reference_answer(ctx, valid) == 0

    free_before = torch.cuda.mem_get_info()[0]
    answers = []
    for ids in (dup, valid, small_oor, small_valid, dup):
        rc, r = _noalloc(ctx, ids)
        assert rc == gb.OK
        answers.append(r)
    free_after = torch.cuda.mem_get_info()[0]
    assert free_after == free_before, "the no-allocation entry point changed free device memory"
    assert answers == [_reference_answer(ctx, ids) for ids in (dup, valid, small_oor, small_valid, dup)]
    assert answers == [2, 0, 1, 0, 2]
    ctx.close()


def test_noalloc_rejects_sizes_beyond_its_maximum():
    ctx = gb.Context(0)
    too_big = torch.zeros(MAX_N + 1, dtype=torch.int32, device="cuda")
    rc, _ = _noalloc(ctx, too_big)
    assert rc == gb.E_OVERFLOW
    assert "GBGPU_NOALLOC_MAX_VERTICES" in gb.library().gbgpu_last_error(ctx.handle).decode()
    ctx.close()
