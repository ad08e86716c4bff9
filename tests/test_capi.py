"""The C-ABI library builds, loads and exports every symbol include/*.h declares (CPU)."""
from __future__ import annotations

import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\*?\s*(ef_[a-z0-9_]+)\s*\(",
                            text, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from eigenfns_gb300 import build as b
    b.build()
    from eigenfns_gb300 import _lib
    return _lib.load()


def test_header_declares_the_boundary():
    names = declared_functions()
    for must in ("ef_op_create", "ef_theta", "ef_precondition", "ef_gram", "ef_rotate",
                 "ef_cheb_step", "ef_kpm_step", "ef_kpm_count_step"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_every_declared_symbol():
    from eigenfns_gb300._lib import SIGNATURES
    assert set(declared_functions()) <= set(SIGNATURES)


def test_status_strings_and_argument_checks_without_gpu(lib):
    import ctypes as C
    assert lib.ef_status_string(0) == b"ok"
    assert lib.ef_version().startswith(b"eigenfns_gb300")
    assert lib.ef_supported_grid(128) == 1 and lib.ef_supported_grid(7) == 0
    # invalid arguments are rejected before any device work
    h = C.c_void_p()
    assert lib.ef_op_create(7, 1.0, 0.0, 0.0, 0.0, None, C.byref(h)) == 1
    assert lib.ef_gram(None, None, 4, 4, 16, None, None, 0, None) == 1
    assert lib.ef_rotate(None, None, None, 0, 4, 16, 0, None) == 1
    assert lib.ef_gram_workspace_bytes(0, 4, 16) == 0


def test_tensor_core_gram_host_checks_without_gpu(lib, monkeypatch):
    """ef_gram_tc rejects misaligned rows, odd K and a short work buffer before any device
    work; with the packed layout on, A^H B with a 32-row B is planned as (B^H A)^H, so both
    orders need the same work buffer."""
    fake_a, fake_b, fake_g, fake_err = 0x10000, 0x20000, 0x30000, 0x40000
    assert lib.ef_gram_tc(fake_a, fake_b + 8, 4, 4, 16, fake_g, fake_err, None, 0, None) == 1
    assert lib.ef_gram_tc(fake_a, fake_b, 4, 4, 15, fake_g, fake_err, None, 0, None) == 1
    assert lib.ef_gram_tc(fake_a, fake_b, 4, 4, 16, fake_g, None, None, 0, None) == 1
    assert lib.ef_gram_tc(fake_a, fake_b, 32, 32, 4096, fake_g, fake_err, fake_g, 16, None) == 4
    K = 2 * 64 ** 3
    monkeypatch.delenv("EF_GRAM_TC_PACK", raising=False)
    for ma in (40, 96, 200):
        assert lib.ef_gram_tc_workspace_bytes(ma, 32, K) == lib.ef_gram_tc_workspace_bytes(32, ma, K)
    monkeypatch.setenv("EF_GRAM_TC_PACK", "0")
    assert lib.ef_gram_tc_workspace_bytes(96, 32, K) > 0
