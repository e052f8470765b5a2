"""CPU-only checks of the C-ABI boundary and the host-side logic (no GPU calls)."""
import ctypes as C
import re

import pytest

from intfadv import _lib, core


def test_library_exports_every_declared_symbol(lib):
    names = _lib.header_functions()
    assert "ia_create" in names and "ia_advect_vof" in names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, f"declared in include/intfadv.h but not exported: {missing}"


def test_every_entry_point_cites_the_reference():
    text = open(_lib.HEADER).read()
    # every declaration except handle plumbing carries a src/<file>.jl citation or says it is new
    for m in re.finditer(r"/\*((?:(?!\*/).)*)\*/\s*\n\s*(?:const\s+)?\w+\**\s+(ia_\w+)\s*\(", text, re.S):
        comment, name = m.group(1), m.group(2)
        if name in ("ia_error_string",):
            continue
        assert ("src/" in comment or "reference" in comment or "no counterpart" in comment
                or "handle" in comment or "stream" in comment or "field" in comment), name


def test_struct_layouts_match_header():
    # sizes computed from the C declarations (x86_64 / aarch64 LP64 ABI)
    assert C.sizeof(_lib.Config) == 4 + 4 + 24 + 8 * 5 + 24 + 4 * 4 + 24 + 8 + 4 + 4
    assert C.sizeof(_lib.Fields) == 15 * 8
    assert C.sizeof(_lib.Status) == 4 + 4 + 16 + 16 + 4 + 8 + 4 + 16 + 8


def test_error_strings(lib):
    assert _lib.error_string(_lib.IA_ERR_NAN).startswith("NaN")
    assert _lib.error_string(_lib.IA_WARN_NOT_CONVERGED).startswith("Poisson")


def test_create_without_device_fails_cleanly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    cfg = core.make_config((8, 8))
    h = C.c_void_p()
    rc = lib.ia_create(C.byref(cfg), C.byref(h))
    assert rc == _lib.IA_ERR_NO_DEVICE and not h.value


def test_config_validation_is_host_side(lib):
    cfg = core.make_config((8, 8))
    cfg.D = 4
    assert lib.ia_create(C.byref(cfg), C.byref(C.c_void_p())) == _lib.IA_ERR_UNSUPPORTED
    cfg = core.make_config((8, 8), exitBC=True)
    assert lib.ia_create(C.byref(cfg), C.byref(C.c_void_p())) == _lib.IA_ERR_UNSUPPORTED
    assert lib.ia_advect_vof(None, None, None, None, 0.1, 1, None) == _lib.IA_ERR_INVALID
    assert lib.ia_poisson_smoother(None, _lib.SMOOTHERS["blocked"]) == _lib.IA_ERR_INVALID
    assert lib.ia_poisson_mg_params(None, 2, 2, 16) == _lib.IA_ERR_INVALID
    assert lib.ia_poisson_mg_relax(None, 1.15) == _lib.IA_ERR_INVALID


def test_split_order_matches_reference():
    from oracle import pyoracle as O
    # dirO = ntuple(i->mod(length(Δt)+i,D)+1, D) (1-based) -> 0-based
    assert O.dir_order(1, 3) == [2, 0, 1]
    assert O.dir_order(2, 3) == [0, 1, 2]
    assert O.dir_order(1, 2) == [0, 1]
    assert O.dir_order(4, 2) == [1, 0]
