"""Discrete adjoint of the time step: gradients of the time-averaged probe-box
kinetic energy with respect to the inlet u-profile and Cs, against central
finite differences of the forward model, and independent of the checkpoint
interval (the backward sweep recomputes each segment exactly)."""
import numpy as np
import pytest

import les_cases
import les_gb300 as G

pytestmark = pytest.mark.gpu

SHAPE = (24, 12, 12)
H = 1.0 / 32
BOX = (2, 10, 2, 10, 2, 10)
STEPS = 6


def _setup(c, profile, seed=4):
    n = int(np.prod(SHAPE))
    c.upload_mask(np.zeros(n, np.uint8))
    c.build_stencil()
    lmax = c.lambda_max(20)
    solid = les_cases.box_mask(SHAPE, (14, 17, 5, 8, 5, 8))
    f = les_cases.init_fields(SHAPE, 0.05, seed)
    c.upload_fields(f)
    c.upload_mask(solid)
    c.set_inlet(profile)
    c.velocity_bcs()
    return lmax


def _params(lmax, cs):
    # mixed precision: the FP64 defect correction reaches a relative residual
    # of 1e-12 where CG on the non-symmetric FP64 system stalls
    return G.step_params(nu=1e-4, rho=les_cases.RHO, cs=cs, dt_fixed=4e-3, solver=G.SOLVER_PCG, rel_tol=1e-12,
                         pcg=G.pcg_opts(precond=G.PC_CHEBYSHEV, max_iter=20000, lambda_min=3 * np.pi ** 2,
                                        lambda_max=lmax, degree=4, precision=G.MIXED, inner_rtol=1e-4))


def _J(profile, cs):
    with G.Context(G.Mesh(*SHAPE, H, H, H)) as c:
        lmax = _setup(c, profile)
        return c.adjoint_forward(_params(lmax, cs), STEPS, STEPS, BOX)


def _grad(profile, cs, every):
    with G.Context(G.Mesh(*SHAPE, H, H, H)) as c:
        lmax = _setup(c, profile)
        J = c.adjoint_forward(_params(lmax, cs), STEPS, every, BOX)
        g, gcs = c.adjoint_backward()
        return J, g, gcs


def _profile():
    rng = np.random.default_rng(9)
    return 1.0 + 0.1 * rng.standard_normal(SHAPE[1] * SHAPE[2])


def test_adjoint_gradient_matches_finite_differences():
    prof, cs = _profile(), 0.17
    J, g, gcs = _grad(prof, cs, 4)
    assert J > 0 and np.all(np.isfinite(g)) and np.isfinite(gcs)
    ny, nz = SHAPE[1], SHAPE[2]
    gi = g.reshape(ny, nz)
    assert np.all(gi[0, :] == 0) and np.all(gi[:, 0] == 0)   # wall cells are not controls
    # the four largest inlet sensitivities and Cs, central differences
    order = np.argsort(-np.abs(g))[:4]
    h = 1e-5
    for idx in order:
        p1, p2 = prof.copy(), prof.copy()
        p1[idx] += h
        p2[idx] -= h
        fd = (_J(p1, cs) - _J(p2, cs)) / (2 * h)
        assert abs(fd - g[idx]) <= 1e-5 * abs(g[idx]), (idx, fd, g[idx])
    hc = 1e-5
    fd = (_J(prof, cs + hc) - _J(prof, cs - hc)) / (2 * hc)
    assert abs(fd - gcs) <= 1e-5 * abs(gcs), (fd, gcs)


def test_adjoint_is_independent_of_the_checkpoint_interval():
    prof, cs = _profile(), 0.15
    J1, g1, c1 = _grad(prof, cs, 1)
    J4, g4, c4 = _grad(prof, cs, 4)
    J6, g6, c6 = _grad(prof, cs, STEPS)
    assert J1 == J4 == J6
    assert np.array_equal(g1, g4) and np.array_equal(g4, g6)
    assert c1 == c4 == c6


def test_tangent_linear_dot_product_test():
    """The FP64 tangent-linear model and the adjoint are exact linearisations
    of the same discrete map: dJ along a random direction equals the
    adjoint gradient projected on it (to the pressure-solve tolerance)."""
    prof, cs = _profile(), 0.17
    rng = np.random.default_rng(31)
    d_in = rng.standard_normal(prof.size)
    d_cs = 0.3
    with G.Context(G.Mesh(*SHAPE, H, H, H)) as c:
        lmax = _setup(c, prof)
        c.adjoint_forward(_params(lmax, cs), STEPS, 4, BOX)
        g, gcs = c.adjoint_backward()
        dJ = c.adjoint_tangent(d_in, d_cs)
    proj = float(np.dot(g, d_in) + gcs * d_cs)
    assert abs(dJ - proj) <= 1e-8 * abs(proj), (dJ, proj)


def test_adjoint_c4_recipe_16_random_entries_64x32x32():
    """The C4 validation recipe on a 64x32x32 grid (h = 1/32, the centred
    obstacle, probe box [48,60)x[8,24)x[8,24), fixed dt from the initial CFL
    value, every pressure solve to relative residual 1e-12, checkpoints every
    8 of 24 steps): the gradient at the uniform inlet u = 1 against central
    finite differences with step 1e-6 on 16 seeded interior inlet entries
    and on Cs, each within 1e-5 relative."""
    shape, h = (64, 32, 32), 1.0 / 32
    n = int(np.prod(shape))
    solid = les_cases.box_mask(shape, (16, 24, 12, 20, 12, 20))
    f = les_cases.init_fields(shape, 0.01, 1234)
    les_cases.velocity_bcs_np(shape, f, solid)
    box = (48, 60, 8, 24, 8, 24)
    nsteps, every, tol, hs = 24, 8, 1e-12, 1e-6
    m = G.Mesh(*shape, h, h, h)

    def run(prof, cs, grad=False):
        with G.Context(m) as c:
            c.upload_mask(np.zeros(n, np.uint8))
            c.build_stencil()
            lmax = c.lambda_max(20)
            c.upload_fields(f)
            c.upload_mask(solid)
            c.set_inlet(prof)
            c.velocity_bcs()
            dt = c.adaptive_dt(les_cases.NU, les_cases.CFL_CONV, les_cases.CFL_VISC, les_cases.DT_MAX)
            prm = G.step_params(nu=les_cases.NU, rho=les_cases.RHO, cs=cs, dt_fixed=dt, solver=G.SOLVER_PCG,
                                rel_tol=tol,
                                pcg=G.pcg_opts(precond=G.PC_CHEBYSHEV, max_iter=50000, lambda_min=3 * np.pi ** 2,
                                               lambda_max=lmax, degree=4, precision=G.MIXED, inner_rtol=1e-4))
            J = c.adjoint_forward(prm, nsteps, every, box, tol)
            return (J,) + c.adjoint_backward() if grad else J

    prof0 = np.ones(shape[1] * shape[2])
    cs0 = les_cases.CS
    J, g, gcs = run(prof0, cs0, grad=True)
    rng = np.random.default_rng(1234)
    cand = [(j, k) for j in range(1, shape[1] - 1) for k in range(1, shape[2] - 1)]
    errs = []
    for q in rng.choice(len(cand), 16, replace=False):
        j, k = cand[q]
        idx = j * shape[2] + k
        p1, p2 = prof0.copy(), prof0.copy()
        p1[idx] += hs
        p2[idx] -= hs
        fd = (run(p1, cs0) - run(p2, cs0)) / (2 * hs)
        errs.append(abs(fd - g[idx]) / abs(g[idx]))
    fdc = (run(prof0, cs0 + hs) - run(prof0, cs0 - hs)) / (2 * hs)
    errs.append(abs(fdc - gcs) / abs(gcs))
    print("C4 recipe at 64x32x32: max relative error %.2e (Cs %.2e)" % (max(errs), errs[-1]))
    assert max(errs) < 1e-5, errs
