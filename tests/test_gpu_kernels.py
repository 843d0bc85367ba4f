"""Per-kernel parity of the CUDA path, through the C ABI, against the golden
fixtures of the compiled reference and against the oracle on larger odd-sized
grids (several thread blocks per axis).  Elementwise and stencil kernels keep
the reference's rounding, so the bar is bit-exact (up to the sign of zero)."""
import numpy as np
import pytest

from conftest import GRIDS, golden_mesh, load_golden, same

import les_gb300 as G
import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=GRIDS)
def g(request):
    return load_golden(request.param)


def ctx_of(m):
    return G.Context(G.Mesh(m.nx, m.ny, m.nz, m.dx, m.dy, m.dz))


def _A(d, tag="A"):
    return {k: d["out_%s_%s" % (tag, k)].copy() for k in O.DIAGS}


def test_velocity_bcs(g):
    m = golden_mesh(g)
    with ctx_of(m) as c:
        for k in "uvw":
            c.upload(k, g["in_" + k])
        c.upload_mask(g["in_solid"])
        c.velocity_bcs()
        for k in "uvw":
            assert same(c.download(k), g["out_vbc_" + k]), k


def test_sgs_nut(g):
    m = golden_mesh(g)
    with ctx_of(m) as c:
        for k in "uvw":
            c.upload(k, g["in_" + k])
        c.upload("nu_t", g["in_nu_t"])
        c.upload_mask(g["in_solid"])
        c.sgs(0.18, want_tau=True)
        assert same(c.download("nu_t"), g["out_sgs_nu_t"])
        assert same(c.download_tau(), g["out_sgs_tau"])
        c.nut_bcs()
        assert same(c.download("nu_t"), g["out_nutbc_nu_t"])
        # fused SGS + BCs equals the two-call sequence
        c.upload("nu_t", g["in_nu_t"])
        c.sgs_nut(0.18)
        assert same(c.download("nu_t"), g["out_nutbc_nu_t"])


def test_momentum(g):
    m = golden_mesh(g)
    dt, nu, rho = (float(x) for x in g["scal"])
    with ctx_of(m) as c:
        for k in "uvw":
            c.upload(k, g["in_" + k])
            c.upload(k + "_new", g["in_%sn" % k])
        c.upload("nu_t", g["out_nutbc_nu_t"])
        c.momentum(dt, nu)
        for k in "uvw":
            assert same(c.download(k), g["out_mom_" + k]), k
            assert same(c.download(k + "_new"), g["out_mom_%sn" % k]), k


def test_correct_velocity_and_dt(g):
    m = golden_mesh(g)
    dt, nu, rho = (float(x) for x in g["scal"])
    with ctx_of(m) as c:
        for k in "uvw":
            c.upload(k, g["in_" + k])
        c.upload("nu_t", g["in_nu_t"])
        assert c.adaptive_dt(nu) == g["out_dt"][0]
        c.upload("p", g["in_p"])
        c.correct_velocity(dt, rho)
        for k in "uvw":
            assert same(c.download(k), g["out_corr_" + k]), k


def test_divergence_and_b(g):
    m = golden_mesh(g)
    dt, nu, rho = (float(x) for x in g["scal"])
    with ctx_of(m) as c:
        for k in "uvw":
            c.upload(k + "_new", g["in_%sn" % k])
        c.upload_mask(g["in_solid"])
        c.divergence(dt, rho)
        assert same(c.download("p_rhs"), g["out_div"])
        c.build_b()
        assert same(c.download("b"), g["out_b"])


def test_pressure_bcs_and_stationary_solvers(g):
    m = golden_mesh(g)
    dt, nu, rho = (float(x) for x in g["scal"])
    with ctx_of(m) as c:
        c.upload_mask(g["in_solid"])
        c.upload("p", g["in_p"])
        c.pressure_bcs()
        assert same(c.download("p"), g["out_pbc_p"])
        for k in "uvw":
            c.upload(k, g["in_" + k])
        c.upload("p", g["in_p"])
        c.solve_jacobi(dt, rho, 100, 1e-6)
        assert same(c.download("p"), g["out_jac_p"])
        c.upload("p", g["in_p"])
        sweeps = c.solve_gs(dt, rho, 30, 1.7, 1e-6)
        assert 1 <= sweeps <= 30
        assert same(c.download("p"), g["out_gs_p"])


def test_stencil_build_and_spmv(g):
    m = golden_mesh(g)
    with ctx_of(m) as c:
        for tag, msk in (("A", g["in_solid"]), ("A0", np.zeros(m.n, np.uint8))):
            c.upload_mask(msk)
            c.build_stencil()
            got = c.get_stencil()
            for k in O.DIAGS:
                assert same(got[k], g["out_%s_%s" % (tag, k)]), (tag, k)
        c.upload_mask(g["in_solid"])
        c.build_stencil()
        c.upload("p", g["in_p"])
        c.spmv("p", "b")
        assert same(c.download("b"), g["out_spmv_q"])
        # stored (arbitrary) matrix gives the same product
        c.set_stencil(_A(g))
        c.spmv("p", "b")
        assert same(c.download("b"), g["out_spmv_q"])
        c.upload("p", g["in_r"])
        c.precond_apply(G.pcg_opts(precond=G.PC_JACOBI), "p", "b")
        assert same(c.download("b"), g["out_jpc_z"])


def test_ic_build_and_apply(g):
    m = golden_mesh(g)
    with ctx_of(m) as c:
        c.set_stencil(_A(g))
        c.build_ic()
        L = c.get_ic_factor()
        for k in O.DIAGS:
            assert same(L[k], g["out_L_" + k]), k
        c.upload("p", g["in_r"])
        c.precond_apply(G.pcg_opts(precond=G.PC_IC), "p", "b")
        assert same(c.download("b"), g["out_icL_z"])
        c.precond_apply(G.pcg_opts(precond=G.PC_IC_A), "p", "b")
        assert same(c.download("b"), g["out_icA_z"])
        # coded matrix (built on the device) gives the same factor
        c.upload_mask(g["in_solid"])
        c.build_stencil()
        c.build_ic()
        L = c.get_ic_factor()
        for k in O.DIAGS:
            assert same(L[k], g["out_L_" + k]), k


def test_lambda_and_chebyshev(g):
    from test_oracle_golden import mt19937_start_vector
    m = golden_mesh(g)
    with ctx_of(m) as c:
        c.upload_mask(np.zeros(m.n, np.uint8))
        c.build_stencil()
        v0 = mt19937_start_vector(m.n)
        lam = c.lambda_max(20, v0)
        # dot products are reassociated: equal to rounding
        assert abs(lam - g["out_lmax"][0]) <= 1e-12 * abs(g["out_lmax"][0])
        assert c.lambda_max(20, None) == lam
        lmax, lmin = (float(x) for x in g["out_lmax"])
        c.upload("p", g["in_r"])
        c.precond_apply(G.pcg_opts(precond=G.PC_CHEBYSHEV, lambda_min=lmin, lambda_max=lmax,
                                   degree=4), "p", "b")
        assert same(c.download("b"), g["out_cheb_z"])


# ---- larger odd-sized grids against the oracle (multi-block tiling edges)

ODD = [(67, 37, 45), (33, 17, 9), (5, 70, 33)]


@pytest.fixture(scope="module", params=ODD, ids=lambda s: "x".join(map(str, s)))
def big(request):
    shape = request.param
    rng = np.random.default_rng(sum(shape))
    n = int(np.prod(shape))
    m = O.Mesh(*shape, 0.021, 0.017, 0.013)
    solid = (rng.random(n) < 0.08).astype(np.uint8)
    d = dict(m=m, solid=solid, u=1 + rng.uniform(-.1, .1, n), v=rng.uniform(-.1, .1, n),
             w=rng.uniform(-.1, .1, n), p=rng.uniform(-1, 1, n), r=rng.uniform(-1, 1, n))
    return d


def test_big_physics_chain(oracle_lib, big):
    m, s = big["m"], big["solid"]
    dt, nu, rho = 1e-4, 1e-5, 1.2
    u, v, w = (big[k].copy() for k in "uvw")
    nt = np.zeros(m.n)
    un, vn, wn = (np.zeros(m.n) for _ in range(3))
    with ctx_of(m) as c:
        for k, a in (("u", u), ("v", v), ("w", w)):
            c.upload(k, a)
        c.upload_mask(s)
        c.sgs_nut(0.17)
        oracle_lib.sgs(m, 0.17, u, v, w, nt)
        oracle_lib.nut_bcs(m, nt, s)
        assert same(c.download("nu_t"), nt)
        c.momentum(dt, nu)
        oracle_lib.momentum(m, dt, nu, u, v, w, nt, un, vn, wn)
        u, un = un, u
        v, vn = vn, v
        w, wn = wn, w
        c.velocity_bcs()
        oracle_lib.velocity_bcs(m, u, v, w, s)
        for k, a in (("u", u), ("v", v), ("w", w), ("u_new", un)):
            assert same(c.download(k), a), k
        c.divergence(dt, rho)
        c.build_b()
        div = np.zeros(m.n)
        b = np.zeros(m.n)
        oracle_lib.divergence(m, dt, rho, un, vn, wn, s, div)
        oracle_lib.build_b(m, div, s, b)
        assert same(c.download("p_rhs"), div)
        assert same(c.download("b"), b)
        c.upload("p", big["p"])
        c.correct_velocity(dt, rho)
        oracle_lib.correct_velocity(m, dt, rho, big["p"], u, v, w)
        for k, a in (("u", u), ("v", v), ("w", w)):
            assert same(c.download(k), a), k


def test_big_pressure_ops(oracle_lib, big):
    m, s = big["m"], big["solid"]
    with ctx_of(m) as c:
        c.upload_mask(s)
        c.build_stencil()
        A = oracle_lib.build_stencil(m, s)
        got = c.get_stencil()
        for k in O.DIAGS:
            assert same(got[k], A[k]), k
        c.upload("p", big["p"])
        c.spmv("p", "b")
        q = np.zeros(m.n)
        oracle_lib.spmv(m, A, big["p"], q)
        assert same(c.download("b"), q)
        c.build_ic()
        L = oracle_lib.ic_build(m, A)
        got = c.get_ic_factor()
        for k in O.DIAGS:
            assert same(got[k], L[k]), k
        c.upload("p", big["r"])
        c.precond_apply(G.pcg_opts(precond=G.PC_IC), "p", "b")
        z = np.zeros(m.n)
        oracle_lib.ic_apply(m, L, big["r"], z)
        assert same(c.download("b"), z)
        c.precond_apply(G.pcg_opts(precond=G.PC_CHEBYSHEV, lambda_min=30.0, lambda_max=2.0e4,
                                   degree=5), "p", "b")
        oracle_lib.cheb_apply(m, A, 30.0, 2.0e4, 5, big["r"], z)
        assert same(c.download("b"), z)
        # pressure BCs and GS-SOR sweeps (wavefront) on the big grid
        c.upload("p", big["p"])
        c.pressure_bcs()
        p = big["p"].copy()
        oracle_lib.pressure_bcs(m, p, s)
        assert same(c.download("p"), p)
        for k in "uvw":
            c.upload(k, big[k])
        c.upload("p", big["p"])
        c.solve_gs(1e-4, 1.2, 7, 1.7, 1e-6)
        p = big["p"].copy()
        oracle_lib.solve_gs(m, 1e-4, 1.2, big["u"], big["v"], big["w"], p, s, 7, 1.7, 1e-6)
        assert same(c.download("p"), p)
        c.upload("p", big["p"])
        c.solve_jacobi(1e-4, 1.2, 9, 1e-6)
        p = big["p"].copy()
        oracle_lib.solve_jacobi(m, 1e-4, 1.2, big["u"], big["v"], big["w"], p, s, 9, 1e-6)
        assert same(c.download("p"), p)


def test_upload_download_many_round_trip():
    """Several slots per call (one synchronisation) move the same bytes as
    one call per slot, and reject a bad slot before copying anything."""
    shape = (9, 7, 5)
    n = int(np.prod(shape))
    rng = np.random.default_rng(3)
    with G.Context(G.Mesh(*shape, 0.1, 0.2, 0.3)) as c:
        src = {k: rng.standard_normal(n) for k in ("u", "v", "w", "p", "nu_t")}
        c.upload_many_ptr({k: v.ctypes.data for k, v in src.items()})
        for k, v in src.items():
            assert same(c.download(k), v), k
        out = {k: np.empty(n) for k in src}
        c.download_many_ptr({k: v.ctypes.data for k, v in out.items()})
        for k in src:
            assert same(out[k], src[k]), k
        with pytest.raises(RuntimeError):
            c.upload_many_ptr({99: src["u"].ctypes.data})
