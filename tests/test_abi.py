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


def _header_enums():
    """name -> value of every enumerator in include/les_gb300.h (implicit
    values counted from the previous one)."""
    import re
    src = open(os.path.join(os.path.dirname(G.PKG), "include", "les_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    out = {}
    for body in re.findall(r"typedef\s+enum\s+\w*\s*\{(.*?)\}", src, flags=re.S):
        nxt = 0
        for item in body.split(","):
            item = item.strip()
            if not item:
                continue
            m = re.match(r"(LES_\w+)\s*(?:=\s*(-?\d+))?$", item)
            assert m, item
            val = int(m.group(2)) if m.group(2) is not None else nxt
            out[m.group(1)] = val
            nxt = val + 1
    return out


def test_binding_constants_match_the_header():
    """The ctypes binding's status, slot, solver, preconditioner, precision
    and option numbers are the header's (no drift when an enumerator is
    added)."""
    e = _header_enums()
    pairs = {"OK": "LES_OK", "NOT_CONVERGED": "LES_NOT_CONVERGED", "NONFINITE": "LES_NONFINITE",
             "BAD_ARG": "LES_BAD_ARG", "CUDA_ERROR": "LES_CUDA_ERROR", "NO_DEVICE": "LES_NO_DEVICE",
             "TIMEOUT": "LES_TIMEOUT",
             "U": "LES_U", "V": "LES_V", "W": "LES_W", "U_NEW": "LES_U_NEW", "V_NEW": "LES_V_NEW",
             "W_NEW": "LES_W_NEW", "P": "LES_P", "P_RHS": "LES_P_RHS", "NU_T": "LES_NU_T", "B": "LES_B",
             "SOLVER_PCG": "LES_SOLVER_PCG", "SOLVER_JACOBI": "LES_SOLVER_JACOBI", "SOLVER_GS": "LES_SOLVER_GS_SOR",
             "PC_JACOBI": "LES_PC_JACOBI", "PC_IC": "LES_PC_IC", "PC_CHEBYSHEV": "LES_PC_CHEBYSHEV",
             "PC_IC_A": "LES_PC_IC_A", "FP64": "LES_FP64", "MIXED": "LES_MIXED"}
    for opt in [k for k in e if k.startswith("LES_OPT_")]:
        pairs[opt[len("LES_"):]] = opt
    missing = [py for py, c in pairs.items() if c not in e]
    assert not missing, missing
    wrong = {py: (getattr(G, py, None), e[c]) for py, c in pairs.items() if getattr(G, py, None) != e[c]}
    assert not wrong, wrong
    assert e["LES_NSLOTS"] == 10
