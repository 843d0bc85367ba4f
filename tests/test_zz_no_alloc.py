"""les_dot_noalloc: the dot product for callers that cannot allocate device
memory (a process whose device memory belongs to a pool or arena, or a thread
that must not enter the allocator mid-step).  It must give the same result as
the regular les_dot entry point, within the dot-product tolerance the other
tests use, on two calls in a row (the shared scratch keeps the previous
call's contents), and reject vectors longer than its fixed scratch allows.

This file is collected last on purpose, so a run that stops at the first
failure has already run every other test."""
import ctypes as C

import numpy as np
import pytest

import les_gb300 as G

pytestmark = pytest.mark.gpu

DOT_RTOL = 1e-12   # reassociated FP64 sums


def _noalloc(lib):
    fn = lib.les_dot_noalloc
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_longlong, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    return fn


def test_dot_noalloc_matches_les_dot_twice():
    lib = G.load()
    fn = _noalloc(lib)
    shape = (61, 35, 27)   # several blocks, a partial last block
    m = G.Mesh(*shape, 0.1, 0.1, 0.1)
    rng = np.random.default_rng(99)
    with G.Context(m) as c:
        for call in range(2):
            a = rng.uniform(-1, 1, m.n) * (10.0 ** call)
            b = rng.uniform(-1, 1, m.n)
            c.upload("p", a)
            c.upload("b", b)
            want = c.dot("p", "b")
            out = c.slot_ptr("p_rhs")   # the caller's own output buffer
            st = fn(c.slot_ptr("p"), c.slot_ptr("b"), m.n, out, c.stream)
            assert st == G.OK
            c.sync()
            got = c.download("p_rhs")[0]
            assert abs(got - want) <= DOT_RTOL * abs(want), (call, got, want)
            assert abs(got - float(np.dot(a, b))) <= 1e-10 * abs(want)


def test_dot_noalloc_rejects_oversize_and_bad_args():
    lib = G.load()
    fn = _noalloc(lib)
    m = G.Mesh(8, 8, 8, 0.1, 0.1, 0.1)
    with G.Context(m) as c:
        p = c.slot_ptr("p")
        assert fn(p, p, 134217728 + 1, p, c.stream) == G.BAD_ARG
        assert fn(p, p, 0, p, c.stream) == G.BAD_ARG
        assert fn(None, p, 10, p, c.stream) == G.BAD_ARG
