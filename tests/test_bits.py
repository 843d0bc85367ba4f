"""FP64 <-> FP32 conversions of the FP32 physics kernels (les_bits.cuh),
compiled for the host and checked against IEEE 754 round-to-nearest-even
conversion (numpy) over the whole FP32 normal range, at ties, and at the
range ends."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "les-model_gb300", "csrc")

SRC = r'''
#include <cstddef>
#include "les_bits.cuh"
extern "C" void to32(const double* in, float* out, size_t n) { for (size_t i = 0; i < n; ++i) out[i] = d2f_bits(in[i]); }
extern "C" void to64(const float* in, double* out, size_t n) { for (size_t i = 0; i < n; ++i) out[i] = f2d_bits(in[i]); }
'''


@pytest.fixture(scope="module")
def bits(tmp_path_factory):
    d = tmp_path_factory.mktemp("bits")
    src, lib = d / "bits.cpp", d / "libbits.so"
    src.write_text(SRC)
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I", CSRC, str(src), "-o", str(lib)],
                   check=True, capture_output=True)
    L = C.CDLL(str(lib))
    L.to32.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t]
    L.to64.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t]

    def to32(x):
        x = np.ascontiguousarray(x, np.float64)
        y = np.empty(x.shape, np.float32)
        L.to32(x.ctypes.data, y.ctypes.data, x.size)
        return y

    def to64(x):
        x = np.ascontiguousarray(x, np.float32)
        y = np.empty(x.shape, np.float64)
        L.to64(x.ctypes.data, y.ctypes.data, x.size)
        return y
    return to32, to64


def same_bits(a, b):
    return np.array_equal(a.view(np.uint32) if a.dtype == np.float32 else a.view(np.uint64),
                          b.view(np.uint32) if b.dtype == np.float32 else b.view(np.uint64))


def test_double_to_float_matches_ieee_nearest_even(bits):
    to32, _ = bits
    rng = np.random.default_rng(5)
    # random significands over the FP32 normal exponent range, both signs
    e = rng.integers(-125, 127, 200000)
    x = rng.uniform(1.0, 2.0, e.size) * np.ldexp(1.0, e) * rng.choice([-1.0, 1.0], e.size)
    with np.errstate(over="ignore"):
        ref = x.astype(np.float32)
    assert same_bits(to32(x), ref)
    # exact ties between neighbouring floats, and one FP64 ulp either side
    f = rng.uniform(1.0, 2.0, 50000).astype(np.float32) * np.float32(2.0) ** rng.integers(-100, 100, 50000)
    f = f.astype(np.float32)
    up = np.nextafter(f, np.float32(np.inf))
    tie = (f.astype(np.float64) + up.astype(np.float64)) / 2.0
    for t in (tie, np.nextafter(tie, -np.inf), np.nextafter(tie, np.inf)):
        assert same_bits(to32(t), t.astype(np.float32))
    # values that round up across a power of two (carry into the exponent)
    top = np.nextafter(np.ldexp(1.0, np.arange(-120, 120)), 0.0)
    assert same_bits(to32(top), top.astype(np.float32))


def test_double_to_float_range_ends(bits):
    to32, _ = bits
    tiny = np.array([0.0, -0.0, 1e-300, -1e-300, 2.0 ** -127, -(2.0 ** -130), 5e-324])
    out = to32(tiny)
    assert np.all(out == 0.0) and np.array_equal(np.signbit(out), np.signbit(tiny))
    big = np.array([1e39, -1e300, np.inf, -np.inf])
    out = to32(big)
    assert np.array_equal(out, np.array([np.inf, -np.inf, np.inf, -np.inf], np.float32))
    assert np.isnan(to32(np.array([np.nan]))).all()
    fmax = float(np.finfo(np.float32).max)
    assert to32(np.array([fmax]))[0] == np.float32(fmax)
    assert to32(np.array([2.0 ** -126]))[0] == np.float32(2.0 ** -126)


def test_float_to_double_exact(bits):
    _, to64 = bits
    rng = np.random.default_rng(6)
    u = rng.integers(0x00800000, 0x7f800000, 200000, dtype=np.uint32) | \
        (rng.integers(0, 2, 200000, dtype=np.uint32) << np.uint32(31))
    f = u.view(np.float32)
    assert same_bits(to64(f), f.astype(np.float64))
    special = np.array([0.0, -0.0, np.inf, -np.inf], np.float32)
    assert same_bits(to64(special), special.astype(np.float64))
    assert np.isnan(to64(np.array([np.nan], np.float32))).all()
    sub = np.array([1e-45, -1e-40], np.float32)   # FP32 subnormals flush to zero
    out = to64(sub)
    assert np.all(out == 0.0) and np.array_equal(np.signbit(out), np.signbit(sub))
