"""ef_gram_noalloc: the Gram entry point that needs no work buffer from its caller.

It exists for callers that cannot hand the library device scratch memory (a
host program that owns only its vectors, or a service whose device-memory budget
forbids allocations after start-up); its split-K partials live in a fixed 8 MiB
array inside the library. This test calls it through the C ABI, twice in a row
with different shapes, and compares each result with ef_gram's. It runs last so
that a failure here leaves every other test already run, and it passes alone in
a fresh process (its first call performs the per-device set-up).
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _gram_with_workspace(lib, A, B):
    ma, K = A.shape
    mb = B.shape[0]
    G = torch.empty((ma, mb), dtype=torch.complex128, device=A.device)
    ws = torch.empty(lib.ef_gram_workspace_bytes(ma, mb, K), dtype=torch.uint8, device=A.device)
    assert lib.ef_gram(A.data_ptr(), B.data_ptr(), ma, mb, K, G.data_ptr(), ws.data_ptr(), ws.numel(),
                       None) == 0
    return G


def _gram_noalloc(lib, A, B):
    ma, K = A.shape
    mb = B.shape[0]
    G = torch.empty((ma, mb), dtype=torch.complex128, device=A.device)
    rc = lib.ef_gram_noalloc(A.data_ptr(), B.data_ptr(), ma, mb, K, G.data_ptr(), None)
    assert rc == 0, lib.ef_last_error()
    return G


def test_gram_noalloc_matches_gram_on_two_calls():
    from eigenfns_gb300 import _lib
    lib = _lib.load()
    g = torch.Generator(device="cuda").manual_seed(11)
    shapes = [(24, 40, 2 * 32 ** 3), (32, 32, 2 * 48 ** 3 + 2)]
    for ma, mb, K in shapes:
        A = torch.randn((ma, K), dtype=torch.complex64, device="cuda", generator=g)
        B = torch.randn((mb, K), dtype=torch.complex64, device="cuda", generator=g)
        ref = _gram_with_workspace(lib, A, B)
        got = _gram_noalloc(lib, A, B)
        torch.cuda.synchronize()
        err = (got - ref).abs().max().item() / ref.abs().max().item()
        assert err < 2e-6, (ma, mb, K, err)


def test_gram_noalloc_rejects_sizes_beyond_its_scratch():
    from eigenfns_gb300 import _lib
    lib = _lib.load()
    A = torch.zeros((1024, 2), dtype=torch.complex64, device="cuda")
    G = torch.empty((1024, 1024), dtype=torch.complex128, device="cuda")
    assert lib.ef_gram_noalloc(A.data_ptr(), A.data_ptr(), 1024, 1024, 2, G.data_ptr(), None) == 6
