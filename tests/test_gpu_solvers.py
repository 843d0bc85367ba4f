"""Solver-level parity: PCG (Jacobi, Chebyshev, IC(L), IC with A as shipped)
in FP64 against the golden fixtures and the oracle, and the mixed-precision
solve against the FP64 solve.

The GPU reduces dot products in a different order from the reference's
sequential sum, so a PCG iterate differs from the reference by rounding that
CG then propagates.  Bars (written per test): x within 1e-10 relative after a
short run; iteration counts within +-1 where the reference converges."""
import numpy as np
import pytest

from conftest import GRIDS, golden_mesh, load_golden, maxrel

import les_cases
import les_gb300 as G
import oracle as O

pytestmark = pytest.mark.gpu

X_RTOL_SHORT = 1e-10    # x after a few iterations
X_RTOL_CONVERGED = 1e-8 # x of a converged solve (tol 1e-8*||b||)


@pytest.fixture(scope="module", params=GRIDS)
def g(request):
    return load_golden(request.param)


def _A(d, tag):
    return {k: d["out_%s_%s" % (tag, k)].copy() for k in O.DIAGS}


VARIANTS = [("shipped", G.PC_IC_A, O.PC_IC, 60), ("cheb", G.PC_CHEBYSHEV, O.PC_CHEB, 300),
            ("jac", G.PC_JACOBI, O.PC_JACOBI, 300), ("icL", G.PC_IC, O.PC_IC, 300)]


def _gpu_pcg(m, A0, L0, b, x0, pc, tol, max_iter, lmin, lmax, precision=G.FP64, **kw):
    with G.Context(G.Mesh(m.nx, m.ny, m.nz, m.dx, m.dy, m.dz)) as c:
        c.upload_mask(np.zeros(m.n, np.uint8))
        c.build_stencil()
        if L0 is not None:
            c.set_ic_factor(L0)
        c.upload("b", b)
        c.upload("p", x0)
        st, r = c.pcg(G.pcg_opts(precond=pc, max_iter=max_iter, tol=tol, lambda_min=lmin,
                                 lambda_max=lmax, degree=4, precision=precision, **kw))
        return st, r, c.download("p")


@pytest.mark.parametrize("variant", VARIANTS, ids=[v[0] for v in VARIANTS])
def test_pcg_short_runs_match_oracle(oracle_lib, g, variant):
    tag, gpc, opc, _ = variant
    m = golden_mesh(g)
    A0 = _A(g, "A0")
    L0 = _A(g, "L0")
    lmax, lmin = (float(x) for x in g["out_lmax"])
    b = g["out_b"]
    tol = float(g["pcg_tol"][0])
    for iters in (1, 5, 12):
        x_ref = g["in_p"].copy()
        Lx = A0 if tag == "shipped" else L0
        it_ref, _ = oracle_lib.pcg(m, A0, b, x_ref, opc, L=Lx, lmin=lmin, lmax=lmax, degree=4,
                                   max_iter=iters, tol=tol)
        # the oracle's own sensitivity to the order of its sums (4 threads
        # instead of 1): the as-shipped preconditioner (A as its own IC
        # factor) amplifies rounding, so its bar scales with that sensitivity
        oracle_lib.set_threads(4)
        x_alt = g["in_p"].copy()
        oracle_lib.pcg(m, A0, b, x_alt, opc, L=Lx, lmin=lmin, lmax=lmax, degree=4, max_iter=iters, tol=tol)
        oracle_lib.set_threads(1)
        bar = max(X_RTOL_SHORT, 10.0 * maxrel(x_alt, x_ref))
        st, r, x = _gpu_pcg(m, A0, L0 if tag == "icL" else None, b, g["in_p"], gpc, tol, iters, lmin, lmax)
        assert r.iters == it_ref
        assert maxrel(x, x_ref) < bar, (tag, iters, maxrel(x, x_ref), bar)


@pytest.mark.parametrize("variant", VARIANTS, ids=[v[0] for v in VARIANTS])
def test_pcg_full_runs_against_golden(g, variant):
    tag, gpc, _, max_iter = variant
    m = golden_mesh(g)
    A0 = _A(g, "A0")
    L0 = _A(g, "L0")
    lmax, lmin = (float(x) for x in g["out_lmax"])
    idx = [v[0] for v in VARIANTS].index(tag)
    it_ref = int(g["out_pcg_iters"][idx])
    st, r, x = _gpu_pcg(m, A0, L0 if tag == "icL" else None, g["out_b"], g["in_p"], gpc,
                        float(g["pcg_tol"][0]), max_iter, lmin, lmax)
    x_ref = g["out_pcg_%s_x" % tag]
    if it_ref < max_iter:   # the reference converged
        assert st == G.OK
        assert abs(r.iters - it_ref) <= 1, (r.iters, it_ref)
        assert maxrel(x, x_ref) < X_RTOL_CONVERGED, maxrel(x, x_ref)
    else:                   # it hit the cap: so must we, ending near the same iterate
        assert r.iters == max_iter and st == G.NOT_CONVERGED
        assert np.all(np.isfinite(x)) == np.all(np.isfinite(x_ref))


def _small_system(seed=5):
    """The small configuration's pressure system after one momentum step."""
    shape, h, solid, f = les_cases.case("small", seed)
    m = G.Mesh(*shape, h, h, h)
    with G.Context(m) as c:
        c.upload_mask(np.zeros(m.n, np.uint8))
        c.build_stencil()
        c.upload_fields(f)
        c.upload_mask(solid)
        c.sgs_nut(les_cases.CS)
        c.momentum(1e-4, les_cases.NU)
        c.velocity_bcs()
        c.divergence(1e-4, les_cases.RHO)
        c.build_b()
        b = c.download("b")
    return m, solid, b


def test_pcg_jacobi_converges_like_oracle_on_small_config(oracle_lib):
    m, solid, b = _small_system()
    om = O.Mesh(m.nx, m.ny, m.nz, m.dx, m.dy, m.dz)
    A0 = oracle_lib.build_stencil(om, np.zeros(m.n, np.uint8))
    tol = 1e-8 * np.linalg.norm(b)
    x_ref = np.zeros(m.n)
    it_ref, _ = oracle_lib.pcg(om, A0, b, x_ref, O.PC_JACOBI, max_iter=1000, tol=tol)
    st, r, x = _gpu_pcg(om, A0, None, b, np.zeros(m.n), G.PC_JACOBI, tol, 1000, 0, 0)
    assert it_ref < 1000 and st == G.OK
    assert abs(r.iters - it_ref) <= 1, (r.iters, it_ref)
    assert maxrel(x, x_ref) < X_RTOL_CONVERGED, maxrel(x, x_ref)


def _lmax(m):
    with G.Context(m) as c:
        c.upload_mask(np.zeros(m.n, np.uint8))
        c.build_stencil()
        return c.lambda_max(20)


@pytest.mark.parametrize("pc", [G.PC_CHEBYSHEV, G.PC_JACOBI])
def test_mixed_precision_matches_fp64(pc):
    """FP32 inner / FP64 defect correction reaches the same relative residual
    1e-8 as the FP64 solve; pressure agrees with the FP64 solution to 1e-6."""
    m, solid, b = _small_system()
    om = O.Mesh(m.nx, m.ny, m.nz, m.dx, m.dy, m.dz)
    tol = 1e-8 * np.linalg.norm(b)
    lmin, lmax = 3 * np.pi ** 2, _lmax(m)
    st64, r64, x64 = _gpu_pcg(om, None, None, b, np.zeros(m.n), pc, tol, 5000, lmin, lmax)
    st32, r32, x32 = _gpu_pcg(om, None, None, b, np.zeros(m.n), pc, tol, 20000, lmin, lmax,
                              precision=G.MIXED, inner_rtol=1e-4)
    assert st64 == G.OK and st32 == G.OK, (st64, st32, r64.iters, r32.iters, r32.outer)
    assert r32.residual < tol
    assert maxrel(x32, x64) < 1e-6, maxrel(x32, x64)


def test_mixed_ic_stalls_like_fp64():
    """CG with the true IC(0) factor does not converge on this non-symmetric
    system (the reference diverges with it too); the mixed path must report
    the same non-convergence with a finite residual no worse than FP64's."""
    m, solid, b = _small_system()
    om = O.Mesh(m.nx, m.ny, m.nz, m.dx, m.dy, m.dz)
    orc = O.Oracle()
    L0 = orc.ic_build(om, orc.build_stencil(om, np.zeros(m.n, np.uint8)))
    tol = 1e-8 * np.linalg.norm(b)
    st64, r64, x64 = _gpu_pcg(om, None, L0, b, np.zeros(m.n), G.PC_IC, tol, 400, 0, 0)
    st32, r32, x32 = _gpu_pcg(om, None, L0, b, np.zeros(m.n), G.PC_IC, tol, 400, 0, 0,
                              precision=G.MIXED, inner_rtol=1e-4)
    assert st64 == G.NOT_CONVERGED and st32 == G.NOT_CONVERGED
    assert np.isfinite(r32.residual) and np.all(np.isfinite(x32))
    assert r32.residual <= 10 * r64.residual


def _odd_system(shape, seed):
    """A random-obstacle system on an odd grid (partial tiles and chunks)."""
    rng = np.random.default_rng(seed)
    n = int(np.prod(shape))
    h = 1.0 / 32
    m = G.Mesh(*shape, h, h, h)
    solid = (rng.random(n) < 0.05).astype(np.uint8)
    f = les_cases.init_fields(shape, 0.05, seed)
    with G.Context(m) as c:
        c.upload_mask(np.zeros(n, np.uint8))
        c.build_stencil()
        lmax = c.lambda_max(20)
        c.upload_fields(f)
        c.upload_mask(solid)
        c.sgs_nut(les_cases.CS)
        c.momentum(1e-4, les_cases.NU)
        c.velocity_bcs()
        c.divergence(1e-4, les_cases.RHO)
        c.build_b()
        b = c.download("b")
    return m, b, lmax


@pytest.mark.parametrize("shape", [(45, 37, 70), (70, 19, 33), (12, 7, 29)], ids=["45x37x70", "70x19x33", "12x7x29"])
@pytest.mark.parametrize("pc,deg", [(G.PC_CHEBYSHEV, 3), (G.PC_CHEBYSHEV, 4), (G.PC_CHEBYSHEV, 5),
                                    (G.PC_CHEBYSHEV, 7), (G.PC_JACOBI, 0)],
                         ids=["cheb3", "cheb4", "cheb5", "cheb7", "jacobi"])
@pytest.mark.parametrize("fused", [1, 2], ids=["columns", "tiles"])
def test_fused_inner_matches_unfused(shape, pc, deg, fused):
    """The fused two-pass FP32 inner iterations (register-column marches and
    shared-memory tiles, both with temporally blocked Chebyshev levels) follow
    the same iteration as the one-kernel-per-operation path: same converged
    solution (pressure within the mixed-vs-FP64 bar, 1e-6 relative) with
    inner iteration counts within 15% (FP32 CG on this non-symmetric system is
    sensitive to rounding: the paths round their inner products differently)."""
    m, b, lmax = _odd_system(shape, sum(shape) + deg)
    tol = 1e-8 * np.linalg.norm(b)
    res = {}
    for mode in (fused, 0):
        with G.Context(m) as c:
            c.set_option(G.OPT_FUSED, mode)
            c.upload_mask(np.zeros(m.n, np.uint8))
            c.build_stencil()
            c.upload("b", b)
            c.upload("p", np.zeros(m.n))
            st, r = c.pcg(G.pcg_opts(precond=pc, max_iter=20000, tol=tol, lambda_min=3 * np.pi ** 2,
                                     lambda_max=lmax, degree=max(deg, 1), precision=G.MIXED, inner_rtol=1e-4))
            res[mode] = (st, r.iters, r.outer, r.residual, c.download("p"))
    (s1, i1, o1, r1, x1), (s0, i0, o0, r0, x0) = res[fused], res[0]
    assert s1 == G.OK and s0 == G.OK, (res[fused][:4], res[0][:4])
    assert r1 < tol and r0 < tol
    assert abs(i1 - i0) <= max(2, 0.15 * i0), (i1, i0)
    assert maxrel(x1, x0) < 1e-6, maxrel(x1, x0)


@pytest.mark.parametrize("shape", [(61, 37, 64), (40, 21, 32)], ids=["61x37x64", "40x21x32"])
@pytest.mark.parametrize("pc,deg", [(G.PC_CHEBYSHEV, 4), (G.PC_CHEBYSHEV, 6), (G.PC_JACOBI, 0)],
                         ids=["cheb4", "cheb6", "jacobi"])
def test_tma_fused_matches_plain_fused(shape, pc, deg):
    """With nz % 16 == 0 the shared-memory tile passes stage their planes with
    TMA; the result must match the same passes with plain loads (identical arithmetic:
    equal iteration counts, pressure equal to rounding of the final outer
    correction) and the unfused path (mixed-vs-FP64 bar)."""
    m, b, lmax = _odd_system(shape, sum(shape) + deg)
    tol = 1e-8 * np.linalg.norm(b)
    res = {}
    for tma, fused in ((1, 2), (0, 2), (0, 0)):
        with G.Context(m) as c:
            c.set_option(G.OPT_FUSED, fused)
            c.set_option(G.OPT_TMA, tma)
            c.upload_mask(np.zeros(m.n, np.uint8))
            c.build_stencil()
            c.upload("b", b)
            c.upload("p", np.zeros(m.n))
            st, r = c.pcg(G.pcg_opts(precond=pc, max_iter=20000, tol=tol, lambda_min=3 * np.pi ** 2,
                                     lambda_max=lmax, degree=max(deg, 1), precision=G.MIXED, inner_rtol=1e-4))
            res[(tma, fused)] = (st, r.iters, r.outer, r.residual, c.download("p"))
    t, f, u = res[(1, 2)], res[(0, 2)], res[(0, 0)]
    assert t[0] == G.OK and f[0] == G.OK and u[0] == G.OK, (t[:4], f[:4], u[:4])
    assert t[1] == f[1] and t[2] == f[2], (t[:4], f[:4])
    assert maxrel(t[4], f[4]) < 1e-12, maxrel(t[4], f[4])
    assert maxrel(t[4], u[4]) < 1e-6, maxrel(t[4], u[4])


def _mixed_solve(m, b, lmax, pc, deg, max_iter, options):
    tol = 1e-8 * np.linalg.norm(b)
    with G.Context(m) as c:
        for opt, val in options:
            c.set_option(opt, val)
        c.upload_mask(np.zeros(m.n, np.uint8))
        c.build_stencil()
        c.upload("b", b)
        c.upload("p", np.zeros(m.n))
        st, r = c.pcg(G.pcg_opts(precond=pc, max_iter=max_iter, tol=tol, lambda_min=3 * np.pi ** 2,
                                 lambda_max=lmax, degree=max(deg, 1), precision=G.MIXED, inner_rtol=1e-4))
        return st, r.iters, r.outer, r.residual, c.download("p")


@pytest.mark.parametrize("fused", [1, 2], ids=["columns", "tiles"])
def test_single_level_chebyshev_follows_unfused(fused):
    """Chebyshev degree 2 (one stencil level; the column pass keeps three
    planes of r' for it) does not converge on these non-symmetric systems in
    any form of the inner iteration, so the fused passes are checked against
    the one-kernel-per-operation path over the first 12 inner iterations: the
    same iterate to FP32 rounding."""
    m, b, lmax = _odd_system((45, 37, 70), 154)
    f = _mixed_solve(m, b, lmax, G.PC_CHEBYSHEV, 2, 12, [(G.OPT_FUSED, fused)])
    u = _mixed_solve(m, b, lmax, G.PC_CHEBYSHEV, 2, 12, [(G.OPT_FUSED, 0)])
    assert f[0] == u[0] == G.NOT_CONVERGED and f[1] == u[1] == 12, (f[:4], u[:4])
    assert np.all(np.isfinite(f[4]))
    assert maxrel(f[4], u[4]) < 1e-4, maxrel(f[4], u[4])


@pytest.mark.parametrize("shape", [(40, 21, 32), (24, 17, 64), (20, 15, 128), (20, 15, 256)],
                         ids=["nz32", "nz64", "nz128", "nz256"])
@pytest.mark.parametrize("pc,deg,rows", [(G.PC_CHEBYSHEV, 4, (0, 0)), (G.PC_CHEBYSHEV, 4, (16, 4)),
                                         (G.PC_CHEBYSHEV, 3, (8, 8)), (G.PC_CHEBYSHEV, 2, (8, 4)),
                                         (G.PC_CHEBYSHEV, 5, (0, 0)), (G.PC_CHEBYSHEV, 7, (0, 0)),
                                         (G.PC_JACOBI, 0, (0, 0))],
                         ids=["cheb4", "cheb4-rows16x4", "cheb3-rows8x8", "cheb2-rows8x4", "cheb5", "cheb7",
                              "jacobi"])
def test_compiled_row_strides_match_runtime_stride(shape, pc, deg, rows):
    """Grids with nz = 32, 64, 128 or 256 run the register-column kernels
    compiled for that row stride (LES_OPT_COL_STRIDE 1, the default); they do
    the arithmetic of the runtime-stride kernels in the same order, so the
    solve is bit-identical: same status, inner and outer iteration counts and
    pressure, for every strip shape (degree 2, which does not converge here,
    over its first 12 inner iterations)."""
    m, b, lmax = _odd_system(shape, sum(shape) + deg)
    cap = 12 if deg == 2 else 20000
    res = {}
    for stride in (1, 0):
        res[stride] = _mixed_solve(m, b, lmax, pc, deg, cap,
                                   [(G.OPT_FUSED, 1), (G.OPT_COL_STRIDE, stride), (G.OPT_ROWS_A, rows[0]),
                                    (G.OPT_ROWS_B, rows[1])])
    a, z = res[1], res[0]
    assert a[0] == (G.NOT_CONVERGED if deg == 2 else G.OK), a[:4]
    assert a[:4] == z[:4], (a[:4], z[:4])
    assert np.array_equal(a[4], z[4])


@pytest.mark.parametrize("cap", [1, 2, 7])
def test_mixed_column_solve_stops_at_the_iteration_cap(cap):
    """The register-column passes test an inner iteration in the pass after
    it (each pass's grid sums are formed by the next one): a mixed solve
    capped at `cap` inner iterations must still stop after exactly `cap` of
    them, report NOT_CONVERGED and leave a finite solution."""
    m, solid, b = _small_system()
    tol = 1e-8 * np.linalg.norm(b)
    with G.Context(m) as c:
        c.set_option(G.OPT_FUSED, 1)
        c.upload_mask(np.zeros(m.n, np.uint8))
        c.build_stencil()
        lmax = c.lambda_max(20)
        c.upload("b", b)
        c.upload("p", np.zeros(m.n))
        st, r = c.pcg(G.pcg_opts(precond=G.PC_CHEBYSHEV, max_iter=cap, tol=tol, lambda_min=3 * np.pi ** 2,
                                 lambda_max=lmax, degree=4, precision=G.MIXED, inner_rtol=1e-4))
        x = c.download("p")
    assert st == G.NOT_CONVERGED and r.iters == cap, (st, r.iters)
    assert np.isfinite(r.residual) and np.all(np.isfinite(x))


def test_wavefront_wait_gives_up_and_the_context_recovers(oracle_lib):
    """Failure path of the pipelined wavefronts, without a GPU fault: with
    LES_OPT_TEST_STALL the first tile withholds its progress, so the tiles
    after it wait on a counter that nothing advances until their bounded
    wait (about 2 s) gives up.  The IC(0)-preconditioned PCG, the IC apply
    and GS-SOR then return LES_TIMEOUT, and with the option off the same
    context computes the reference's results bit for bit again."""
    import time

    shape, h = (24, 40, 36), 1.0 / 16   # several tiles along j and k
    m = G.Mesh(*shape, h, h, h)
    om = O.Mesh(*shape, h, h, h)
    n = m.n
    rng = np.random.default_rng(8)
    solid = np.zeros(n, np.uint8)
    u, v, w = (rng.uniform(-1, 1, n) for _ in range(3))
    p0 = rng.uniform(-1, 1, n)
    r = rng.uniform(-1, 1, n)
    A = oracle_lib.build_stencil(om, solid)
    L = oracle_lib.ic_build(om, A)
    with G.Context(m) as c:
        c.upload_mask(solid)
        c.build_stencil()
        c.build_ic()
        ic = G.pcg_opts(precond=G.PC_IC, max_iter=3)
        c.set_option(G.OPT_TEST_STALL, 1)
        t0 = time.perf_counter()
        c.upload("b", r)
        with pytest.raises(G.LesError) as e:
            c.precond_apply(ic, "b", "p_rhs")
        assert e.value.status == G.TIMEOUT
        c.upload("p", np.zeros(n))
        with pytest.raises(G.LesError) as e:
            c.pcg(ic)
        assert e.value.status == G.TIMEOUT
        for k, a in (("u", u), ("v", v), ("w", w), ("p", p0)):
            c.upload(k, a)
        with pytest.raises(G.LesError) as e:
            c.solve_gs(1e-4, 1.2, 5, 1.7, 0.0)
        assert e.value.status == G.TIMEOUT
        assert time.perf_counter() - t0 < 60
        # the same context, option off: bit-exact again
        c.set_option(G.OPT_TEST_STALL, 0)
        c.upload("b", r)
        c.precond_apply(ic, "b", "p_rhs")
        z = np.zeros(n)
        oracle_lib.ic_apply(om, L, r, z)
        assert np.array_equal(c.download("p_rhs"), z)
        c.upload("p", p0)
        sweeps = c.solve_gs(1e-4, 1.2, 5, 1.7, 0.0)
        pr = p0.copy()
        it = oracle_lib.solve_gs(om, 1e-4, 1.2, u, v, w, pr, solid, 5, 1.7, 0.0)
        assert sweeps == it == 5
        assert np.array_equal(c.download("p"), pr)
