"""The C ABI library loads and exports every entry point include/les_gb300.h
declares; without a GPU it refuses to create a context instead of falling
back to the CPU.  No compute calls are made here."""
import ctypes as C
import os

import pytest

import les_gb300 as G


def _lib():
    if not os.path.exists(G.LIB_PATH):
        pytest.skip("libles_gb300.so not built (run __graft_entry__.build())")
    return G.load()


def test_header_declares_entry_points():
    names = G.exported_symbols()
    assert len(names) >= 35
    for must in ("les_create", "les_step", "les_pcg", "les_solve_gs", "les_build_ic", "les_spmv"):
        assert must in names


def test_library_exports_every_declared_symbol():
    lib = _lib()
    missing = [n for n in G.exported_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_abi_version_and_status_strings():
    lib = _lib()
    assert lib.les_abi_version() == 1
    for s in range(7):
        assert lib.les_status_string(s)


def test_bad_arguments_rejected_before_any_device_work():
    lib = _lib()
    h = C.c_void_p()
    # meshes below 3 cells per axis or with non-positive spacing are refused
    for m in (G.Mesh(2, 8, 8, 0.1, 0.1, 0.1), G.Mesh(8, 8, 8, 0.0, 0.1, 0.1)):
        assert lib.les_create(C.byref(m), 0, C.byref(h)) == G.BAD_ARG
    assert lib.les_create(None, 0, C.byref(h)) == G.BAD_ARG


def test_no_cpu_fallback_without_gpu():
    lib = _lib()
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    m = G.Mesh(8, 8, 8, 0.1, 0.1, 0.1)
    assert lib.les_create(C.byref(m), 0, C.byref(h)) == G.NO_DEVICE
    with pytest.raises(G.LesError):
        G.Context(m)
