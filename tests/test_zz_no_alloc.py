"""The allocation-free vector assembly (elfel_sysvec_assemble_noalloc).

It serves callers that cannot allocate device memory where they assemble; its
scratch is a fixed array inside the library.  This file is collected last so
that a run stopping at the first failure has run every other test first.

The device inputs and output here are PyTorch tensors (memory the caller owns);
the results are compared with the allocating entry point elfel_sysvec_assemble
on two calls in a row.  Tolerance: none -- both add the same values in the
same order, so the results must be equal bit for bit (the tolerance of the
other COO-mode tests).
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(ctx, nrow, rows_dev, vals_dev, out_dev):
    import torch

    torch.cuda.synchronize()  # the inputs were written on PyTorch's stream
    return ctx.lib.elfel_sysvec_assemble_noalloc(ctx.h, nrow, ctypes.c_void_p(rows_dev.data_ptr()),
                                                 ctypes.c_void_p(vals_dev.data_ptr()), rows_dev.numel(),
                                                 ctypes.c_void_p(out_dev.data_ptr()))


def _reference(E, ctx, nrow, rows, vals):
    out = np.zeros(nrow)
    rows = np.ascontiguousarray(rows, dtype=np.int64)
    vals = np.ascontiguousarray(vals, dtype=np.float64)
    ctx.check(ctx.lib.elfel_sysvec_assemble(ctx.h, nrow, E._native.ptr(rows, E._native._i64p),
                                            E._native.ptr(vals), rows.shape[0], E._native.ptr(out)))
    return out


def test_noalloc_matches_allocating_entry_point(E, gpu):
    import torch

    ctx = gpu
    rng = np.random.default_rng(2026)
    for call, (nrow, n) in enumerate([(50_000, 400_000), (7_001, 90_000)]):
        rows = rng.integers(1, nrow + 1, n)
        rows[: n // 50] = 3  # one long row (sorted in global memory)
        vals = rng.standard_normal(n)
        # signed zeros: rows 1 and 2 receive only -0.0 (the sum is +0, as in
        # SysvecAssembler, which adds into zeros(T, n)); the first entry of row
        # 5 is -0.0 and the others cancel to zero
        rows[rows == 1] = 4
        rows[rows == 2] = 4
        rows[rows == 5] = 6
        rows[-6:] = [1, 1, 2, 5, 5, 5]
        vals[-6:] = [-0.0, -0.0, -0.0, -0.0, 1.5, -1.5]
        expected = _reference(E, ctx, nrow, rows, vals)
        assert np.signbit(expected[0]) == 0 and np.signbit(expected[1]) == 0
        rows_d = torch.from_numpy(rows).cuda()
        vals_d = torch.from_numpy(vals).cuda()
        out_d = torch.full((nrow,), float("nan"), dtype=torch.float64, device="cuda")
        ctx.check(_noalloc(ctx, nrow, rows_d, vals_d, out_d))
        got = out_d.cpu().numpy()
        # bit for bit, signed zeros included
        assert np.array_equal(got.view(np.int64), expected.view(np.int64)), f"call {call}"


def test_noalloc_limits_and_errors(E, gpu):
    import torch

    ctx = gpu
    limit = 524288  # ELFEL_NOALLOC_MAX_ROWS
    rows_d = torch.ones(4, dtype=torch.int64, device="cuda")
    vals_d = torch.ones(4, dtype=torch.float64, device="cuda")
    out_d = torch.zeros(limit + 1, dtype=torch.float64, device="cuda")
    rc = _noalloc(ctx, limit + 1, rows_d, vals_d, out_d)
    assert rc == E._native.ELFEL_ERR_ARG
    assert "exceed" in ctx.lib.elfel_ctx_last_error(ctx.h).decode()
    bad = torch.tensor([1, 9, 2], dtype=torch.int64, device="cuda")  # row 9 > nrow = 5
    out_d[:5] = 7.0
    rc = _noalloc(ctx, 5, bad, vals_d[:3].contiguous(), out_d)
    assert rc == E._native.ELFEL_ERR_ARG
    assert (out_d[:5].cpu() == 7.0).all(), "out must stay unchanged when a row is out of range"
    # entries but no rows: every row number is out of range
    rc = _noalloc(ctx, 0, rows_d, vals_d, out_d)
    assert rc == E._native.ELFEL_ERR_ARG
    assert "no rows" in ctx.lib.elfel_ctx_last_error(ctx.h).decode()
    empty = torch.empty(0, dtype=torch.int64, device="cuda")
    assert _noalloc(ctx, 0, empty, torch.empty(0, dtype=torch.float64, device="cuda"), out_d) == 0
