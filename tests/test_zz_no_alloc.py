"""The allocation-free solve (ntg_chol_solve_noalloc) against the workspace solve.

Callers that cannot allocate device memory at the call site (an XLA FFI
handler, which only receives the buffers XLA allocated; a server whose device
memory is all reserved up front in its own pool) use
ntg_chol_solve_noalloc, whose refinement workspace is a fixed device array of
the library. This test calls it through the C ABI twice in a row, on two
different right-hand sides, and compares each result with ntg_chol_solve run
with a caller workspace. It lives in its own file, collected last.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _spd(n, seed):
    rng = np.random.default_rng(seed)
    g = rng.standard_normal((n, n + 3)).astype(np.float32)
    return torch.from_numpy((g @ g.T / n).astype(np.float32)).cuda()


def test_noalloc_solve_matches_workspace_solve_twice(nt):
    from nt_gb300 import _lib as L
    lib = L.load()
    n, m = 300, 10
    k = _spd(n, 0)
    fac = torch.empty_like(k)
    lam = torch.zeros(2, dtype=torch.float64, device='cuda')
    info = torch.zeros(1, dtype=torch.int32, device='cuda')
    L.call('ntg_chol_factor', L.stream(), k.data_ptr(), n, 1e-3, 0, fac.data_ptr(),
           lam.data_ptr(), info.data_ptr())
    assert int(info.item()) == 0
    ws_bytes = int(lib.ntg_chol_workspace_bytes(n, m))
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device='cuda')
    for call in range(2):
        b = torch.randn((n, m), generator=torch.Generator().manual_seed(call)).cuda()
        ref = torch.empty_like(b)
        got = torch.full_like(b, float('nan'))
        r_ref = torch.zeros(1, dtype=torch.float64, device='cuda')
        r_got = torch.zeros(1, dtype=torch.float64, device='cuda')
        L.call('ntg_chol_solve', L.stream(), k.data_ptr(), fac.data_ptr(), lam.data_ptr(), n,
               b.data_ptr(), m, ref.data_ptr(), 2, ws.data_ptr(), ws_bytes, r_ref.data_ptr())
        rc = lib.ntg_chol_solve_noalloc(ctypes.c_void_p(L.stream()), k.data_ptr(),
                                        fac.data_ptr(), lam.data_ptr(), n, b.data_ptr(), m,
                                        got.data_ptr(), 2, r_got.data_ptr())
        assert rc == 0, lib.ntg_last_error().decode()
        torch.cuda.synchronize()
        # same arithmetic on the same inputs: equal within the float32 tolerance of the suite
        torch.testing.assert_close(got, ref, rtol=1e-6, atol=1e-7)
        torch.testing.assert_close(r_got, r_ref, rtol=1e-6, atol=1e-12)


def test_noalloc_rejects_sizes_beyond_the_fixed_scratch(nt):
    from nt_gb300 import _lib as L
    lib = L.load()
    rc = lib.ntg_chol_solve_noalloc(None, None, None, None, 100000, None, 100, None, 2, None)
    assert rc == 1
    assert b'too large for the fixed scratch' in lib.ntg_last_error()
