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


_CHILD = r"""
import ctypes as C, json, sys
sys.path[:0] = sys.argv[1:]
import torch
import les_gb300 as G
lib = G.load()
fn = lib.les_dot_noalloc
fn.argtypes = [C.c_void_p, C.c_void_p, C.c_longlong, C.c_void_p, C.c_void_p]
fn.restype = C.c_int
n = 1 << 20
g = torch.Generator(device="cuda").manual_seed(5)
a = torch.rand(n, dtype=torch.float64, device="cuda", generator=g) - 0.5
b = torch.rand(n, dtype=torch.float64, device="cuda", generator=g) - 0.5
out = torch.zeros(4, dtype=torch.float64, device="cuda")
want = float(torch.dot(a, b))
torch.cuda.synchronize()
free = [torch.cuda.mem_get_info()[0]]
for q in range(3):
    st = fn(a.data_ptr(), b.data_ptr(), n, out[q:].data_ptr(), None)
    assert st == 0, st
    torch.cuda.synchronize()
    free.append(torch.cuda.mem_get_info()[0])
got = [float(x) for x in out[:3].cpu()]
print(json.dumps({"free": free, "got": got, "want": want}))
"""


def test_dot_noalloc_reserves_nothing_after_its_first_call():
    """In a fresh process: the first call on the device loads the module that
    holds the scratch array (CUDA's lazy loading); every later call leaves the
    device's free memory exactly as it was."""
    import json
    import os
    import subprocess
    import sys

    here = os.path.dirname(os.path.abspath(__file__))
    pkg = os.path.join(os.path.dirname(here), "les-model_gb300")
    r = subprocess.run([sys.executable, "-c", _CHILD, os.path.join(pkg, "py"), pkg], capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    free = res["free"]
    assert free[2] == free[1] and free[3] == free[1], free
    for got in res["got"]:
        assert abs(got - res["want"]) <= 1e-10 * abs(res["want"]), (got, res["want"])
