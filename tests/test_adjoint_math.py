"""CPU checks of the identity the adjoint pressure solve rests on: the
reference's pressure matrix (as the oracle builds it from src/pressure.cpp)
is non-symmetric only through its Neumann rows with doubled coefficients, and
S = W A is symmetric for W = 1/2 per mirrored axis (inlet plane, j walls, k
walls; 1 on the decoupled outlet rows).  Then A^-T g = W A^-1 (W^-1 g)."""
import numpy as np
import pytest

import oracle as O


def _weights(nx, ny, nz):
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    w = np.where(i == 0, 0.5, 1.0)
    w = w * np.where((j == 0) | (j == ny - 1), 0.5, 1.0)
    w = w * np.where((k == 0) | (k == nz - 1), 0.5, 1.0)
    w = np.where(i == nx - 1, 1.0, w)
    return w.reshape(-1)


def _dense(m, A):
    nx, ny, nz = m.nx, m.ny, m.nz
    n = nx * ny * nz
    M = np.zeros((n, n))
    off = {"c": (0, 0, 0), "e": (1, 0, 0), "w": (-1, 0, 0), "n": (0, 1, 0), "s": (0, -1, 0),
           "t": (0, 0, 1), "b": (0, 0, -1)}
    for i in range(nx):
        for j in range(ny):
            for k in range(nz):
                r = (i * ny + j) * nz + k
                for d, (di, dj, dk) in off.items():
                    a = A[d][r]
                    ii, jj, kk = i + di, j + dj, k + dk
                    if 0 <= ii < nx and 0 <= jj < ny and 0 <= kk < nz:
                        M[r, (ii * ny + jj) * nz + kk] += a
                    else:
                        assert a == 0.0 or d == "c"
    return M


@pytest.mark.parametrize("shape,h", [((7, 5, 6), (0.1, 0.1, 0.1)), ((9, 4, 8), (0.05, 0.11, 0.07))])
def test_pressure_matrix_is_symmetrisable(oracle_lib, shape, h):
    m = O.Mesh(*shape, *h)
    A = oracle_lib.build_stencil(m, np.zeros(m.n, np.uint8))
    M = _dense(m, A)
    w = _weights(*shape)
    S = w[:, None] * M
    assert np.max(np.abs(M - M.T)) > 0          # A itself is not symmetric
    assert np.max(np.abs(S - S.T)) <= 1e-14 * np.max(np.abs(S))
    # the adjoint solve: A^T y = g  <=>  y = W A^-1 (W^-1 g)
    g = np.random.default_rng(1).standard_normal(m.n)
    y = w * np.linalg.solve(M, g / w)
    assert np.max(np.abs(M.T @ y - g)) <= 1e-10 * np.max(np.abs(g))
