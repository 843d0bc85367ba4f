"""The Chebyshev preconditioner of the mixed-precision column passes is the
reference's polynomial (les-model src/pressure.cpp:851-906) evaluated in
three-term form: with pc_{k-1} = (z_{k-1} - z_{k-2}) / a_{k-1} (z_{-1} = 0),
level k is z_k = (1 + g_k) z_{k-1} - g_k z_{k-2} + a_k (r - A z_{k-1}),
g_k = a_k b_k / a_{k-1}, with the reference's a_k and b_k.  CPU only: the
identity in FP64 against the oracle's two-term apply on the pressure matrix
the column passes serve (built before the obstacle), and the per-level
weights in the form the kernels use them (A's plane-uniform coefficients
folded in, level 1 on r', level 2's z_0 term joined to its r term)."""
import math

import numpy as np
import pytest

import oracle as O


def _ab(lmin, lmax, degree):
    """a_0 and (a_k, b_k), k = 1 .. degree-1, as the reference forms them."""
    d = (lmax + lmin) / 2.0
    c = (lmax - lmin) / 2.0
    a = 2.0 / d
    out = []
    for _ in range(1, degree):
        b = (c * a / 2.0) * (c * a / 2.0)
        a_new = 1.0 / (d - b)
        out.append((a_new, b))
        a = a_new
    return 2.0 / d, out


def _three_term(spmv, r, lmin, lmax, degree):
    a0, ab = _ab(lmin, lmax, degree)
    zm2 = np.zeros_like(r)
    zm1 = a0 * r
    ap = a0
    for a, b in ab:
        g = a * b / ap
        z = (1.0 + g) * zm1 - g * zm2 + a * (r - spmv(zm1))
        zm2, zm1, ap = zm1, z, a
    return zm1


@pytest.fixture(scope="module")
def case(oracle_lib):
    shape, h = (11, 7, 6), 1.0 / 8
    m = O.Mesh(*shape, h, h, h)
    A = oracle_lib.build_stencil(m, np.zeros(m.n, np.uint8))
    r = np.random.default_rng(5).standard_normal(m.n)

    def spmv(p):
        q = np.zeros(m.n)
        oracle_lib.spmv(m, A, p, q)
        return q

    lmin = 3 * math.pi ** 2
    lmax = 2.0 * float(np.max(A["c"]))
    return m, A, r, spmv, lmin, lmax


@pytest.mark.parametrize("degree", [2, 3, 4, 5, 7])
def test_three_term_form_is_the_reference_polynomial(oracle_lib, case, degree):
    m, A, r, spmv, lmin, lmax = case
    z_ref = np.zeros(m.n)
    oracle_lib.cheb_apply(m, A, lmin, lmax, degree, r, z_ref)
    z = _three_term(spmv, r, lmin, lmax, degree)
    assert np.max(np.abs(z - z_ref)) <= 1e-12 * np.max(np.abs(z_ref))


def test_folded_level_weights(oracle_lib, case):
    """Per-level weights as the kernels apply them: z_k = cc zc + cx (zw + ze)
    + cy (zs + zn) + cz (zb + zt) + rr r' + gg z_{k-2}, from A's interior
    coefficients (c0, x1, y1, z1).  Checked on the interior cells of a field,
    where the 7-point stencil has its base coefficients."""
    m, A, r, spmv, lmin, lmax = case
    nx, ny, nz = m.shape
    centre = (nx // 2) * ny * nz + (ny // 2) * nz + nz // 2   # an interior cell
    c0, x1, y1, z1 = (float(A[k][centre]) for k in ("c", "w", "s", "b"))
    assert c0 > 0 and x1 < 0 and y1 < 0 and z1 < 0
    a0, ab = _ab(lmin, lmax, 4)
    rr_ = np.random.default_rng(9).standard_normal((12, 11, 10))

    def stencil(f, cc, cx, cy, cz):
        o = np.zeros_like(f)
        o[1:-1, 1:-1, 1:-1] = (cc * f[1:-1, 1:-1, 1:-1]
                               + cx * (f[:-2, 1:-1, 1:-1] + f[2:, 1:-1, 1:-1])
                               + cy * (f[1:-1, :-2, 1:-1] + f[1:-1, 2:, 1:-1])
                               + cz * (f[1:-1, 1:-1, :-2] + f[1:-1, 1:-1, 2:]))
        return o

    def apply_a(f):
        return stencil(f, c0, x1, y1, z1)

    # reference recurrence on the interior (both forms read the same ring of
    # neighbours; cells deeper than the degree from the boundary are exact)
    z, p = a0 * rr_, rr_.copy()
    for a, b in ab:
        res = rr_ - apply_a(z)
        p = res + b * p
        z = z + a * p
    # folded weights
    zm2, zm1, ap = None, None, a0
    for k, (a, b) in enumerate(ab, start=1):
        g = a * b / ap
        sc = a0 if k == 1 else 1.0
        cc = sc * (1.0 + g) - a * sc * c0
        if k == 1:
            cc += a
        src = rr_ if k == 1 else zm1
        zk = stencil(src, cc, -a * sc * x1, -a * sc * y1, -a * sc * z1)
        if k == 2:
            zk = zk + (a - g * a0) * rr_
        elif k >= 3:
            zk = zk + a * rr_ - g * zm2
        zm2, zm1, ap = (a0 * rr_ if k == 1 else zm1), zk, a
    inner = (slice(3, -3),) * 3
    assert np.max(np.abs(zm1[inner] - z[inner])) <= 1e-12 * np.max(np.abs(z[inner]))
