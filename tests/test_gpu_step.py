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


def _oracle_threads():
    import os
    return max(1, os.cpu_count() or 1)


def _config_params(precond, lmax=0.0):
    prm_o = O.StepParams(nu=les_cases.NU, rho=les_cases.RHO, cs=les_cases.CS, cfl_conv=les_cases.CFL_CONV,
                         cfl_visc=les_cases.CFL_VISC, dt_max=les_cases.DT_MAX, solver=0,
                         pc={G.PC_JACOBI: O.PC_JACOBI, G.PC_CHEBYSHEV: O.PC_CHEB}[precond],
                         max_iter=10000, tol=0.0, rel_tol=1e-8, omega=1.7, lmin=3 * np.pi ** 2, lmax=lmax,
                         degree=4, dt_fixed=-1.0)
    prm = G.step_params(nu=les_cases.NU, rho=les_cases.RHO, cs=les_cases.CS, cfl_conv=les_cases.CFL_CONV,
                        cfl_visc=les_cases.CFL_VISC, dt_max=les_cases.DT_MAX, solver=G.SOLVER_PCG,
                        rel_tol=1e-8, pcg=G.pcg_opts(precond=precond, max_iter=10000, lambda_min=3 * np.pi ** 2,
                                                     lambda_max=lmax, degree=4))
    return prm_o, prm


def test_small_config_100_steps_match_oracle():
    """The small configuration as specified: 64x32x32, Jacobi-PCG to relative
    residual 1e-8, all 100 steps, against the oracle (src/main.cpp:108-165),
    both trajectories run independently from the same initial state.  Every
    step: dt identical, iteration counts within +-1, u, v, w, p, nu_t within
    1e-10 relative; the mask bit-exact at the end."""
    shape, h, solid, f = les_cases.case("small", 11)
    m = G.Mesh(*shape, h, h, h)
    om = O.Mesh(*shape, h, h, h)
    n = m.n
    orc = O.Oracle()
    orc.set_threads(_oracle_threads())
    A0 = orc.build_stencil(om, np.zeros(n, np.uint8))
    of = {k: v.copy() for k, v in f.items()}
    of["solid"] = solid
    prm_o, prm = _config_params(G.PC_JACOBI)
    worst = 0.0
    with G.Context(m) as c:
        c.upload_mask(np.zeros(n, np.uint8))
        c.build_stencil()
        c.upload_mask(solid)
        c.upload_fields(f)
        for step in range(100):
            s = c.step(prm)
            it, dt = orc.step(om, of, A0, None, prm_o)
            assert s.status == G.OK, (step, s.status)
            assert s.dt == dt, (step, s.dt, dt)
            assert abs(s.iters - it) <= 1, (step, s.iters, it)
            out = c.download_fields(("u", "v", "w", "p", "nu_t"))
            for k in ("u", "v", "w", "p", "nu_t"):
                e = maxrel(out[k], of[k])
                worst = max(worst, e)
                assert e < FIELD_RTOL, (step, k, e)
        assert same(c.download_mask(), solid)
    print("100 steps: worst relative field difference %.2e" % worst)


@pytest.mark.parametrize("precond", [G.PC_CHEBYSHEV, G.PC_JACOBI], ids=["cheb4", "jacobi"])
def test_large_fp64_step_matches_oracle(precond):
    """The plain FP64 path at 256x128x128 (the obstacle scaled 4x): the first
    time step with Chebyshev(4)-PCG (lambda_max from the reference's power
    iteration) and with Jacobi-PCG, to relative residual 1e-8, against the
    oracle on all host cores: fields within 1e-10 relative, iteration counts
    within +-1."""
    shape, h, solid, f = les_cases.case("large", 1234)
    m = G.Mesh(*shape, h, h, h)
    om = O.Mesh(*shape, h, h, h)
    n = m.n
    orc = O.Oracle()
    orc.set_threads(_oracle_threads())
    A0 = orc.build_stencil(om, np.zeros(n, np.uint8))
    lmax_o = orc.lambda_max(om, A0, O.mt19937_start_vector(n), 20) if precond == G.PC_CHEBYSHEV else 0.0
    with G.Context(m) as c:
        c.upload_mask(np.zeros(n, np.uint8))
        c.build_stencil()
        lmax = c.lambda_max(20) if precond == G.PC_CHEBYSHEV else 0.0
        assert abs(lmax - lmax_o) <= 1e-12 * lmax_o
        c.upload_mask(solid)
        c.upload_fields(f)
        prm_o, prm = _config_params(precond, lmax)
        s = c.step(prm)
        out = c.download_fields(("u", "v", "w", "p", "nu_t"))
    of = {k: v.copy() for k, v in f.items()}
    of["solid"] = solid
    prm_o.lmax = lmax
    it, dt = orc.step(om, of, A0, None, prm_o)
    assert s.status == G.OK and s.dt == dt
    assert abs(s.iters - it) <= 1, (s.iters, it)
    for k in ("u", "v", "w", "p", "nu_t"):
        assert maxrel(out[k], of[k]) < FIELD_RTOL, (k, maxrel(out[k], of[k]))


def test_mixed_trajectory_128x64x64_pressure_error():
    """The mixed-precision step (FP32 inner Chebyshev(4)-PCG in FP64 defect
    correction, FP32 nu_t and momentum tendencies) against the plain FP64 step
    over 24 steps of a 128x64x64 case with the centred obstacle, both to
    relative residual 1e-8, beside a run whose every solve is converged to
    relative residual 1e-12.  Every step: u, v, w within 1e-7 and p within
    1e-6 of the FP64 run, and the mixed pressure within 1e-6 of the
    converged one."""
    shape, h, solid, f = les_cases.case("adjoint", 5)
    m = G.Mesh(*shape, h, h, h)
    n = m.n
    runs = {}
    for name in ("mixed", "fp64", "conv"):
        c = G.Context(m)
        c.upload_mask(np.zeros(n, np.uint8))
        c.build_stencil()
        lmax = c.lambda_max(20)
        c.upload_mask(solid)
        c.upload_fields(f)
        prec = G.FP64 if name == "fp64" else G.MIXED
        opts = G.pcg_opts(precond=G.PC_CHEBYSHEV, max_iter=50000 if prec == G.MIXED else 10000,
                          lambda_min=3 * np.pi ** 2, lambda_max=lmax, degree=4, precision=prec, inner_rtol=1e-4,
                          inner_max_iter=5000, max_outer=40)
        prm = G.step_params(nu=les_cases.NU, rho=les_cases.RHO, cs=les_cases.CS, cfl_conv=les_cases.CFL_CONV,
                            cfl_visc=les_cases.CFL_VISC, dt_max=les_cases.DT_MAX, solver=G.SOLVER_PCG,
                            rel_tol=1e-12 if name == "conv" else 1e-8, pcg=opts)
        if name == "conv":
            c.set_option(G.OPT_PHYS32, 0)
        runs[name] = (c, prm)
    rows = []
    try:
        for step in range(24):
            st = {k: c.step(p) for k, (c, p) in runs.items()}
            for k, x in st.items():
                assert x.status == G.OK, (step, k, x.status)
            d = {k: runs[k][0].download_fields(("u", "v", "w", "p")) for k in runs}
            e = {q: maxrel(d["mixed"][q], d["fp64"][q]) for q in ("u", "v", "w", "p")}
            e["p_mixed_conv"] = maxrel(d["mixed"]["p"], d["conv"]["p"])
            e["p_fp64_conv"] = maxrel(d["fp64"]["p"], d["conv"]["p"])
            rows.append(e)
    finally:
        for c, _ in runs.values():
            c.close()
    print("max over steps:", {k: "%.2e" % max(r[k] for r in rows) for k in rows[0]})
    for step, e in enumerate(rows):
        for q in ("u", "v", "w"):
            assert e[q] < 1e-7, (step, q, e)
        assert e["p"] < 1e-6, (step, e)
        assert e["p_mixed_conv"] < 1e-6, (step, e)


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


IO_IN = ("u", "v", "w", "u_new", "v_new", "w_new", "p", "nu_t")
IO_OUT = ("u", "v", "w", "u_new", "v_new", "w_new", "p", "p_rhs", "nu_t")


@pytest.mark.parametrize("graph,precision", [(1, G.MIXED), (0, G.MIXED), (0, G.FP64)],
                         ids=["graph-mixed", "launches-mixed", "launches-fp64"])
def test_step_io_matches_separate_calls(graph, precision):
    """les_step_io (upload, step, download in one call; the downloads of
    u_new, v_new, w_new, nu_t and p_rhs overlap the pressure solve, released
    by an event after the step's physics) gives what les_upload_many +
    les_step + les_download_many give, bit for bit, every step -- the host's
    fields fed back into the next step as a drop-in host loop does."""
    shape = (64, 32, 32)
    n = int(np.prod(shape))
    solid = les_cases.box_mask(shape, (16, 20, 10, 14, 10, 14))
    f = les_cases.init_fields(shape, 0.01, 77)
    h = 1.0 / 32
    m = G.Mesh(*shape, h, h, h)
    with G.Context(m) as c:
        c.upload_mask(np.zeros(n, np.uint8))
        c.build_stencil()
        lmax = c.lambda_max(20)
    prm = G.step_params(nu=les_cases.NU, rho=les_cases.RHO, cs=les_cases.CS, cfl_conv=les_cases.CFL_CONV,
                        solver=G.SOLVER_PCG, rel_tol=1e-8,
                        pcg=G.pcg_opts(precond=G.PC_CHEBYSHEV, max_iter=5000, lambda_min=3 * np.pi ** 2,
                                       lambda_max=lmax, degree=4, precision=precision, inner_rtol=1e-4))
    host = [{k: np.zeros(n) for k in IO_OUT} for _ in range(2)]
    ctxs = []
    try:
        for hb in host:
            c = G.Context(m)
            ctxs.append(c)
            c.set_option(G.OPT_GRAPH, graph)
            c.upload_mask(np.zeros(n, np.uint8))
            c.build_stencil()
            c.upload_fields(f)
            c.upload_mask(solid)
            c.velocity_bcs()
            for k in IO_OUT:
                hb[k][:] = c.download(k)
        for step in range(5):
            a, b = ctxs
            ha, hb = host
            a.upload_many_ptr({k: ha[k].ctypes.data for k in IO_IN})
            sa = a.step(prm)
            for k in IO_OUT:
                a.download_ptr(k, ha[k].ctypes.data)
            sb, ms = b.step_io(prm, {k: hb[k].ctypes.data for k in IO_IN}, {k: hb[k].ctypes.data for k in IO_OUT})
            assert ms > 0
            assert (sa.dt, sa.iters, sa.outer, sa.residual, sa.status) == (sb.dt, sb.iters, sb.outer, sb.residual,
                                                                          sb.status), step
            for k in IO_OUT:
                assert same(ha[k], hb[k]), (step, k)
    finally:
        for c in ctxs:
            c.close()


def test_step_io_rejects_bad_arguments_before_copying():
    """les_step_io checks its arguments before it copies anything: a bad
    solver, slot or null host pointer returns LES_BAD_ARG with the context's
    fields untouched."""
    shape = (24, 12, 12)
    n = int(np.prod(shape))
    h = 1.0 / 32
    with G.Context(G.Mesh(*shape, h, h, h)) as c:
        c.upload_mask(np.zeros(n, np.uint8))
        c.build_stencil()
        u0 = np.linspace(0.0, 1.0, n)
        c.upload("u", u0)
        junk = np.full(n, 7.0)
        bad = G.step_params(nu=les_cases.NU, rho=les_cases.RHO, cs=les_cases.CS, solver=9)
        with pytest.raises(G.LesError):
            c.step_io(bad, {"u": junk.ctypes.data}, {})
        good = G.step_params(nu=les_cases.NU, rho=les_cases.RHO, cs=les_cases.CS, solver=G.SOLVER_JACOBI)
        with pytest.raises(G.LesError):
            c.step_io(good, {"u": junk.ctypes.data, 99: junk.ctypes.data}, {})
        with pytest.raises(G.LesError):
            c.step_io(good, {"u": junk.ctypes.data, "v": 0}, {})
        assert same(c.download("u"), u0)


def test_step_io_gs_sor_and_partial_outputs():
    """les_step_io with the GS-SOR solver (nothing downloads early) and with a
    subset of the fields in and out: the same fields as separate calls."""
    shape = (40, 24, 32)
    n = int(np.prod(shape))
    solid = les_cases.box_mask(shape, (10, 14, 8, 12, 10, 14))
    f = les_cases.init_fields(shape, 0.01, 5)
    h = 1.0 / 32
    m = G.Mesh(*shape, h, h, h)
    prm = G.step_params(nu=les_cases.NU, rho=les_cases.RHO, cs=les_cases.CS, cfl_conv=les_cases.CFL_CONV,
                        solver=G.SOLVER_GS, omega=1.7, stat_max_iter=60, stat_tol=1e-6)
    ins, outs = ("u", "v", "w", "p"), ("p", "nu_t", "u_new")
    host = [{k: np.zeros(n) for k in set(ins) | set(outs)} for _ in range(2)]
    ctxs = []
    try:
        for hb in host:
            c = G.Context(m)
            ctxs.append(c)
            c.upload_mask(np.zeros(n, np.uint8))
            c.build_stencil()
            c.upload_fields(f)
            c.upload_mask(solid)
            c.velocity_bcs()
            for k in hb:
                hb[k][:] = c.download(k)
        for step in range(3):
            a, b = ctxs
            ha, hb = host
            a.upload_many_ptr({k: ha[k].ctypes.data for k in ins})
            sa = a.step(prm)
            for k in outs:
                a.download_ptr(k, ha[k].ctypes.data)
            sb, ms = b.step_io(prm, {k: hb[k].ctypes.data for k in ins}, {k: hb[k].ctypes.data for k in outs})
            assert (sa.iters, sa.status) == (sb.iters, sb.status), step
            for k in outs:
                assert same(ha[k], hb[k]), (step, k)
    finally:
        for c in ctxs:
            c.close()


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
