"""Whole time steps (les_step) against the reference trajectories in the golden
fixtures and against the oracle on the small configuration.

Stationary solvers (Jacobi, GS-SOR) contain no dot products, so their
trajectories are bit-exact.  PCG trajectories differ by reassociated dot
products; the bar is 1e-10 relative per step on u, v, w, p and nu_t and
iteration counts within +-1 for runs that converge."""
import numpy as np
import pytest

from conftest import GRIDS, golden_mesh, load_golden, maxrel, same

import les_cases
import les_gb300 as G
import oracle as O

pytestmark = pytest.mark.gpu

FIELD_RTOL = 1e-10

# golden trajectory index -> (solver, precond)
TRAJ = {0: (G.SOLVER_PCG, G.PC_IC_A), 1: (G.SOLVER_PCG, G.PC_JACOBI), 2: (G.SOLVER_PCG, G.PC_IC),
        3: (G.SOLVER_PCG, G.PC_CHEBYSHEV), 4: (G.SOLVER_JACOBI, 0), 5: (G.SOLVER_GS, 0)}


@pytest.fixture(scope="module", params=GRIDS)
def g(request):
    return load_golden(request.param)


@pytest.mark.parametrize("traj", sorted(TRAJ))
def test_golden_trajectory(g, traj):
    m = golden_mesh(g)
    dt, nu, rho = (float(x) for x in g["scal"])
    solver, pc = TRAJ[traj]
    lmax, lmin = (float(x) for x in g["out_lmax"])
    with G.Context(G.Mesh(m.nx, m.ny, m.nz, m.dx, m.dy, m.dz)) as c:
        c.upload_mask(np.zeros(m.n, np.uint8))
        c.build_stencil()   # main.cpp order: A (and L) before the mask
        c.build_ic()
        c.upload_mask(g["in_solid"])
        f = dict(u=g["in_u"], v=g["in_v"], w=g["in_w"], u_new=g["in_un"], v_new=g["in_vn"],
                 w_new=g["in_wn"], p=np.zeros(m.n), p_rhs=np.zeros(m.n), nu_t=np.zeros(m.n))
        c.upload_fields(f)
        c.velocity_bcs()
        its = []
        for step in range(3):
            prm = G.step_params(nu=nu, rho=rho, cs=0.18, dt_fixed=(0.0 if step == 2 else dt),
                                solver=solver, rel_tol=1e-8 if solver == G.SOLVER_PCG else 0.0,
                                stat_max_iter=100 if solver == G.SOLVER_JACOBI else 40,
                                pcg=G.pcg_opts(precond=pc, max_iter=200, lambda_min=lmin,
                                               lambda_max=lmax, degree=4))
            s = c.step(prm)
            assert s.dt == g["traj%d_dt" % traj][step]
            its.append(s.iters)
        out = c.download_fields()
    keys = (("u", "u"), ("v", "v"), ("w", "w"), ("p", "p"), ("nu_t", "nu_t"), ("u_new", "un"))
    if solver != G.SOLVER_PCG:
        for k, gk in keys + (("p_rhs", "p_rhs"),):
            assert same(out[k], g["traj%d_%s" % (traj, gk)]), k
        return
    ref_its = list(g["traj%d_iters" % traj])
    for a, b in zip(its, ref_its):
        if b < 200:
            assert abs(a - b) <= 1, (its, ref_its)
        else:
            assert a == 200, (its, ref_its)
    if all(b < 200 for b in ref_its):
        for k, gk in keys:
            assert maxrel(out[k], g["traj%d_%s" % (traj, gk)]) < FIELD_RTOL, k


def test_small_config_steps_match_oracle(oracle_lib):
    """Five steps of the small configuration (64x32x32, Jacobi-PCG to 1e-8
    relative) against the oracle, step by step."""
    shape, h, solid, f = les_cases.case("small", 11)
    m = G.Mesh(*shape, h, h, h)
    om = O.Mesh(*shape, h, h, h)
    n = m.n
    A0 = oracle_lib.build_stencil(om, np.zeros(n, np.uint8))
    of = {k: v.copy() for k, v in f.items()}
    of["solid"] = solid
    prm_o = O.StepParams(nu=les_cases.NU, rho=les_cases.RHO, cs=les_cases.CS, cfl_conv=les_cases.CFL_CONV,
                         cfl_visc=les_cases.CFL_VISC, dt_max=les_cases.DT_MAX, solver=0, pc=O.PC_JACOBI,
                         max_iter=1000, tol=0.0, rel_tol=1e-8, omega=1.7, lmin=0, lmax=0, degree=4,
                         dt_fixed=-1.0)
    prm = G.step_params(nu=les_cases.NU, rho=les_cases.RHO, cs=les_cases.CS, cfl_conv=les_cases.CFL_CONV,
                        cfl_visc=les_cases.CFL_VISC, dt_max=les_cases.DT_MAX, solver=G.SOLVER_PCG,
                        rel_tol=1e-8, pcg=G.pcg_opts(precond=G.PC_JACOBI, max_iter=1000))
    with G.Context(m) as c:
        c.upload_mask(np.zeros(n, np.uint8))
        c.build_stencil()
        c.upload_mask(solid)
        c.upload_fields(f)
        for step in range(5):
            s = c.step(prm)
            it, dt = oracle_lib.step(om, of, A0, None, prm_o)
            assert s.dt == dt
            assert abs(s.iters - it) <= 1, (step, s.iters, it)
            out = c.download_fields(("u", "v", "w", "p", "nu_t"))
            for k in ("u", "v", "w", "p", "nu_t"):
                assert maxrel(out[k], of[k]) < FIELD_RTOL, (step, k, maxrel(out[k], of[k]))
        assert same(c.download_mask(), solid)


def _mixed_run(shape, solid, f, lmax, steps, graph, fused=1, dt_fixed=0.0, pdl=1):
    h = 1.0 / 32
    m = G.Mesh(*shape, h, h, h)
    with G.Context(m) as c:
        c.set_option(G.OPT_GRAPH, graph)
        c.set_option(G.OPT_FUSED, fused)
        c.set_option(G.OPT_PDL, pdl)
        c.upload_mask(np.zeros(m.n, np.uint8))
        c.build_stencil()
        c.upload_fields(f)
        c.upload_mask(solid)
        c.velocity_bcs()
        prm = G.step_params(nu=les_cases.NU, rho=les_cases.RHO, cs=les_cases.CS, cfl_conv=les_cases.CFL_CONV,
                            dt_fixed=dt_fixed, solver=G.SOLVER_PCG, rel_tol=1e-8,
                            pcg=G.pcg_opts(precond=G.PC_CHEBYSHEV, max_iter=5000, lambda_min=3 * np.pi ** 2,
                                           lambda_max=lmax, degree=4, precision=G.MIXED, inner_rtol=1e-4))
        stats = []
        for _ in range(steps):
            s = c.step(prm)
            stats.append((s.dt, s.iters, s.outer, s.residual, s.status))
        return stats, c.download_fields()


@pytest.mark.parametrize("shape,fused,dt_fixed", [((64, 32, 32), 1, 0.0), ((45, 37, 70), 1, 1e-4),
                                                  ((40, 21, 32), 2, 0.0)],
                         ids=["64x32x32-columns", "45x37x70-columns-fixed-dt", "40x21x32-tiles"])
def test_graph_step_matches_launch_by_launch(shape, fused, dt_fixed):
    """The time step replayed as one CUDA graph (device dt, both solver loops
    as conditional nodes, one graph per velocity-buffer parity) runs exactly
    the kernels of the launch-by-launch step in the same order: identical
    fields and statistics, over enough steps to reuse both parities."""
    rng = np.random.default_rng(sum(shape))
    n = int(np.prod(shape))
    solid = les_cases.box_mask(shape, (shape[0] // 4, shape[0] // 4 + 4, shape[1] // 3, shape[1] // 3 + 4,
                                       shape[2] // 3, shape[2] // 3 + 4))
    f = les_cases.init_fields(shape, 0.01, int(rng.integers(1 << 30)))
    h = 1.0 / 32
    with G.Context(G.Mesh(*shape, h, h, h)) as c:
        c.upload_mask(np.zeros(n, np.uint8))
        c.build_stencil()
        lmax = c.lambda_max(20)
    s0, f0 = _mixed_run(shape, solid, f, lmax, 5, 0, fused, dt_fixed)
    s1, f1 = _mixed_run(shape, solid, f, lmax, 5, 1, fused, dt_fixed)
    assert s0 == s1, (s0, s1)
    for k in ("u", "v", "w", "p", "nu_t", "u_new", "p_rhs"):
        assert same(f0[k], f1[k]), k


@pytest.mark.parametrize("graph", [0, 1], ids=["launches", "graph"])
def test_dependent_launch_changes_nothing(graph):
    """The column passes as programmatic dependent launches (each waits for
    the grid before it ahead of its first memory access) give bit-identical
    steps to plain stream order, launch by launch and inside the step graph."""
    shape = (48, 40, 36)
    n = int(np.prod(shape))
    solid = les_cases.box_mask(shape, (12, 16, 12, 18, 10, 16))
    f = les_cases.init_fields(shape, 0.01, 77)
    h = 1.0 / 32
    with G.Context(G.Mesh(*shape, h, h, h)) as c:
        c.upload_mask(np.zeros(n, np.uint8))
        c.build_stencil()
        lmax = c.lambda_max(20)
    s0, f0 = _mixed_run(shape, solid, f, lmax, 4, graph, pdl=0)
    s1, f1 = _mixed_run(shape, solid, f, lmax, 4, graph, pdl=1)
    assert s0 == s1, (s0, s1)
    for k in ("u", "v", "w", "p", "nu_t"):
        assert same(f0[k], f1[k]), k


def test_fp32_physics_step_close_to_fp64_physics():
    """nu_t and the momentum update in FP32 (LES_OPT_PHYS32, the mixed path's
    default) against the reference-order FP64 kernels, both with the mixed
    pressure solve: same solver work, and velocity, pressure and nu_t within
    the FP32 rounding of the tendencies (the velocity update itself is FP64)."""
    shape = (64, 32, 32)
    n = int(np.prod(shape))
    solid = les_cases.box_mask(shape, (16, 24, 12, 20, 12, 20))
    f = les_cases.init_fields(shape, 0.01, 1234)
    h = 1.0 / 32
    with G.Context(G.Mesh(*shape, h, h, h)) as c:
        c.upload_mask(np.zeros(n, np.uint8))
        c.build_stencil()
        lmax = c.lambda_max(20)
    res = {}
    for p32 in (0, 1):
        m = G.Mesh(*shape, h, h, h)
        with G.Context(m) as c:
            c.set_option(G.OPT_PHYS32, p32)
            c.upload_mask(np.zeros(n, np.uint8))
            c.build_stencil()
            c.upload_fields(f)
            c.upload_mask(solid)
            c.velocity_bcs()
            prm = G.step_params(nu=les_cases.NU, rho=les_cases.RHO, cs=les_cases.CS, cfl_conv=les_cases.CFL_CONV,
                                solver=G.SOLVER_PCG, rel_tol=1e-8,
                                pcg=G.pcg_opts(precond=G.PC_CHEBYSHEV, max_iter=5000, lambda_min=3 * np.pi ** 2,
                                               lambda_max=lmax, degree=4, precision=G.MIXED, inner_rtol=1e-4))
            stats = [c.step(prm) for _ in range(6)]
            res[p32] = (stats, c.download_fields(("u", "v", "w", "p", "nu_t")))
    (s0, f0), (s1, f1) = res[0], res[1]
    for a, b in zip(s0, s1):
        assert a.status == G.OK and b.status == G.OK
        assert abs(a.iters - b.iters) <= 2, (a.iters, b.iters)
        assert abs(a.dt - b.dt) <= 1e-6 * a.dt
    for k, bar in (("u", 1e-7), ("v", 1e-7), ("w", 1e-7), ("p", 1e-6), ("nu_t", 1e-4)):
        scale = max(np.max(np.abs(f0[k])), 1e-300)
        err = np.max(np.abs(f1[k] - f0[k])) / scale
        assert err < bar, (k, err)
