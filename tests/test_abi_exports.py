"""The C-ABI library loads without a GPU and exports every entry point that
include/issm.h declares (no compute calls)."""
import ctypes
import os
import re

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "issm.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(issm_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "issm_mixture_logdensity" in syms and "issm_resample_systematic" in syms
    assert len(syms) >= 25


def test_library_exports_every_declared_symbol(issm):
    path = issm.native.library_path()
    if not os.path.exists(path):
        pytest.skip("libissm103.so not built (run __graft_entry__.build())")
    lib = ctypes.CDLL(path)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert missing == []


def test_bindings_cover_header(issm):
    bound = {name for name, _, _ in issm.native.SIGNATURES}
    assert set(declared_symbols()) <= bound


def test_version_and_status_strings(issm):
    if not os.path.exists(issm.native.library_path()):
        pytest.skip("libissm103.so not built")
    lib = issm.native.load()
    assert lib.issm_version().decode().startswith("issm103")
    assert "zero" in lib.issm_status_string(-5).decode()
    assert "workspace" in lib.issm_status_string(-7).decode()


def test_argument_errors_need_no_gpu(issm):
    """Validation happens before any launch: NULL and size errors return
    negative codes without touching a device."""
    if not os.path.exists(issm.native.library_path()):
        pytest.skip("libissm103.so not built")
    lib = issm.native.load()
    assert lib.issm_failure_reset(None, None) == -1
    assert lib.issm_fill_normals(1, 0, -1, None, 0, None) == -2
    assert lib.issm_fill_normals(1, 0, 4, None, 0, None) == -1
    assert lib.issm_fill_normals(1, 0, 4, 1234, 7, None) == -3
    assert lib.issm_gather(None, 0, 1, None, 1, 0, None, None) == -2
    b = issm.native.Bank(0, 1, 0, 0, 0, 0, 1, 1, 1, None, None)
    den = issm.native.Denominator(0, 0, 1, None)
    assert lib.issm_mixture_logdensity(ctypes.byref(b), ctypes.byref(den), 1, 1, None, 0, 1, None, None, 0, 0,
                                       None) == -2
    b.dim = 2
    b.family = 1  # Student-t without dofs
    assert lib.issm_mixture_logdensity(ctypes.byref(b), ctypes.byref(den), 1, 1, None, 0, 1, None, None, 0, 0,
                                       None) == -1
    assert lib.issm_resample_systematic(1, 4, 0, 1.5, 4, 1, 1, 10 ** 6, None) == -2


def test_run_descriptor_layout_matches_binding(issm):
    """The ctypes mirror of issm_amis_run_desc has the C struct's size and
    field offsets; a NULL descriptor is rejected before any launch."""
    if not os.path.exists(issm.native.library_path()):
        pytest.skip("libissm103.so not built")
    lib = issm.native.load()
    D = issm.native.AmisRunDesc
    assert ctypes.sizeof(D) == lib.issm_amis_run_desc_bytes()
    assert D.workspace_bytes.offset == lib.issm_amis_run_desc_workspace_offset()
    assert lib.issm_amis_run(None, None) == -1
    assert lib.issm_amis_run_workspace_bytes(0, 10, 4) == 0
    # a history without its arrays is rejected before any launch
    tgt = issm.native.Target(0, 4, 0, 0, None, None, None, 0.0, 0.0)
    sizes = (ctypes.c_int64 * 2)(10, 10)
    desc = D()
    desc.history = issm.native.Bank(4, 2, 0, issm.native.SCALE_FACTOR, 0, 0, None, None, None, None, None, None)
    desc.target = ctypes.cast(ctypes.byref(tgt), ctypes.c_void_p)
    desc.rounds = 2
    desc.round_sizes = ctypes.cast(sizes, ctypes.c_void_p)
    assert lib.issm_amis_run(ctypes.byref(desc), None) == -1
    desc.history.count = 1  # fewer history slots than rounds
    assert lib.issm_amis_run(ctypes.byref(desc), None) == -2


def test_draw_philox_argument_errors_need_no_gpu(issm):
    if not os.path.exists(issm.native.library_path()):
        pytest.skip("libissm103.so not built")
    lib = issm.native.load()
    b = issm.native.Bank(2, 1, 0, issm.native.SCALE_FACTOR, 0, 0, 1, 1, 1, None, None, None)
    assert lib.issm_draw_philox(ctypes.byref(b), 0, 1, None, 0, None, 0, None, 0, 0, None, None, 0, None) == 0
    assert lib.issm_draw_philox(ctypes.byref(b), 0, 1, None, 0, None, 0, None, 0, -1, 1, None, 0, None) == -2
    assert lib.issm_draw_philox(ctypes.byref(b), 0, 1, None, 0, None, 0, None, 0, 4, None, None, 0, None) == -1
    assert lib.issm_draw_philox(ctypes.byref(b), 1, 1, None, 0, None, 0, None, 0, 4, 1, None, 0, None) == -2
    b.family = 1  # Student-t needs radial normals
    assert lib.issm_draw_philox(ctypes.byref(b), 0, 1, None, 0, None, 0, None, 0, 4, 1, None, 0, None) == -1
