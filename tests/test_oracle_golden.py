"""The oracle (oracle/les_oracle.c) against the golden fixtures produced by
the compiled reference.  CPU only.  Everything is bit-exact: the oracle runs
on one thread, in the reference's operation order, without FMA."""
import math

import numpy as np
import pytest

from conftest import GRIDS, golden_mesh, load_golden, same

import oracle as O
from oracle import mt19937_start_vector  # noqa: F401  (also used by the GPU tests)


@pytest.fixture(scope="module", params=GRIDS)
def g(request):
    return load_golden(request.param)


def _A(d, tag="A"):
    return {k: d["out_%s_%s" % (tag, k)].copy() for k in O.DIAGS}


def test_velocity_bcs(oracle_lib, g):
    m = golden_mesh(g)
    a = [g["in_" + k].copy() for k in "uvw"]
    oracle_lib.velocity_bcs(m, *a, g["in_solid"])
    for k, x in zip("uvw", a):
        assert same(x, g["out_vbc_" + k])


def test_sgs_and_nut_bcs(oracle_lib, g):
    m = golden_mesh(g)
    nt = g["in_nu_t"].copy()
    tau = np.zeros(6 * m.n)
    oracle_lib.sgs(m, 0.18, g["in_u"], g["in_v"], g["in_w"], nt, tau)
    assert same(nt, g["out_sgs_nu_t"])
    assert same(tau, g["out_sgs_tau"])
    oracle_lib.nut_bcs(m, nt, g["in_solid"])
    assert same(nt, g["out_nutbc_nu_t"])


def test_momentum(oracle_lib, g):
    m = golden_mesh(g)
    dt, nu, rho = (float(x) for x in g["scal"])
    outs = [g["in_" + k].copy() for k in ("un", "vn", "wn")]
    oracle_lib.momentum(m, dt, nu, g["in_u"], g["in_v"], g["in_w"], g["out_nutbc_nu_t"], *outs)
    # after the reference's swap, f.u holds the new values
    for k, x in zip("uvw", outs):
        assert same(x, g["out_mom_" + k])
    for k in "uvw":
        assert same(g["in_" + k], g["out_mom_%sn" % k])


def test_correct_velocity(oracle_lib, g):
    m = golden_mesh(g)
    dt, nu, rho = (float(x) for x in g["scal"])
    a = [g["in_" + k].copy() for k in "uvw"]
    oracle_lib.correct_velocity(m, dt, rho, g["in_p"], *a)
    for k, x in zip("uvw", a):
        assert same(x, g["out_corr_" + k])


def test_adaptive_dt(oracle_lib, g):
    m = golden_mesh(g)
    dt, nu, rho = (float(x) for x in g["scal"])
    got = oracle_lib.adaptive_dt(m, g["in_u"], g["in_v"], g["in_w"], g["in_nu_t"], nu)
    assert got == g["out_dt"][0]


def test_pressure_bcs_and_stationary(oracle_lib, g):
    m = golden_mesh(g)
    dt, nu, rho = (float(x) for x in g["scal"])
    p = g["in_p"].copy()
    oracle_lib.pressure_bcs(m, p, g["in_solid"])
    assert same(p, g["out_pbc_p"])
    p = g["in_p"].copy()
    oracle_lib.solve_jacobi(m, dt, rho, g["in_u"], g["in_v"], g["in_w"], p, g["in_solid"])
    assert same(p, g["out_jac_p"])
    p = g["in_p"].copy()
    oracle_lib.solve_gs(m, dt, rho, g["in_u"], g["in_v"], g["in_w"], p, g["in_solid"], 30)
    assert same(p, g["out_gs_p"])


def test_divergence_and_b(oracle_lib, g):
    m = golden_mesh(g)
    dt, nu, rho = (float(x) for x in g["scal"])
    div = np.zeros(m.n)
    oracle_lib.divergence(m, dt, rho, g["in_un"], g["in_vn"], g["in_wn"], g["in_solid"], div)
    assert same(div, g["out_div"])
    b = np.zeros(m.n)
    oracle_lib.build_b(m, div, g["in_solid"], b)
    assert same(b, g["out_b"])


def test_stencil_spmv_precond(oracle_lib, g):
    m = golden_mesh(g)
    A = oracle_lib.build_stencil(m, g["in_solid"])
    for k in O.DIAGS:
        assert same(A[k], g["out_A_" + k]), k
    A0 = oracle_lib.build_stencil(m, np.zeros(m.n, np.uint8))
    for k in O.DIAGS:
        assert same(A0[k], g["out_A0_" + k]), k
    q = np.zeros(m.n)
    oracle_lib.spmv(m, A, g["in_p"], q)
    assert same(q, g["out_spmv_q"])
    z = np.zeros(m.n)
    oracle_lib.jacobi_precond(A, g["in_r"], z)
    assert same(z, g["out_jpc_z"])


def test_ic(oracle_lib, g):
    m = golden_mesh(g)
    A, A0 = _A(g), _A(g, "A0")
    L = oracle_lib.ic_build(m, A)
    for k in O.DIAGS:
        assert same(L[k], g["out_L_" + k]), k
    L0 = oracle_lib.ic_build(m, A0)
    for k in O.DIAGS:
        assert same(L0[k], g["out_L0_" + k]), k
    z = np.zeros(m.n)
    oracle_lib.ic_apply(m, L, g["in_r"], z)
    assert same(z, g["out_icL_z"])
    z = np.zeros(m.n)
    oracle_lib.ic_apply(m, A, g["in_r"], z)
    assert same(z, g["out_icA_z"])


def test_lambda_and_chebyshev(oracle_lib, g):
    m = golden_mesh(g)
    A0 = _A(g, "A0")
    v0 = mt19937_start_vector(m.n)
    lmax = oracle_lib.lambda_max(m, A0, v0, 20)
    assert lmax == g["out_lmax"][0]
    assert g["out_lmax"][1] == 3.0 * math.pi ** 2
    z = np.zeros(m.n)
    oracle_lib.cheb_apply(m, A0, g["out_lmax"][1], lmax, 4, g["in_r"], z)
    assert same(z, g["out_cheb_z"])


def test_pcg_variants(oracle_lib, g):
    m = golden_mesh(g)
    A, A0 = _A(g), _A(g, "A0")
    L0 = {k: g["out_L0_" + k] for k in O.DIAGS}
    b = g["out_b"]
    tol = float(g["pcg_tol"][0])
    lmax, lmin = (float(x) for x in g["out_lmax"])
    want = list(g["out_pcg_iters"])
    cases = [("shipped", O.PC_IC, A0, 60), ("cheb", O.PC_CHEB, None, 300),
             ("jac", O.PC_JACOBI, None, 300), ("icL", O.PC_IC, L0, 300)]
    for (tag, pc, L, mi), it_ref in zip(cases, want):
        x = g["in_p"].copy()
        it, _ = oracle_lib.pcg(m, A0, b, x, pc, L=L, lmin=lmin, lmax=lmax, degree=4,
                               max_iter=mi, tol=tol)
        assert it == it_ref, tag
        assert same(x, g["out_pcg_%s_x" % tag]), tag


SOLVERS = {0: (0, O.PC_IC, "A"), 1: (0, O.PC_JACOBI, None), 2: (0, O.PC_IC, "L"),
           3: (0, O.PC_CHEB, None), 4: (1, 0, None), 5: (2, 0, None)}


@pytest.mark.parametrize("solver", sorted(SOLVERS))
def test_trajectory(oracle_lib, g, solver):
    m = golden_mesh(g)
    dt, nu, rho = (float(x) for x in g["scal"])
    A0 = _A(g, "A0")
    L0 = {k: g["out_L0_" + k] for k in O.DIAGS}
    lmax, lmin = (float(x) for x in g["out_lmax"])
    kind, pc, fac = SOLVERS[solver]
    f = dict(u=g["in_u"].copy(), v=g["in_v"].copy(), w=g["in_w"].copy(), u_new=g["in_un"].copy(),
             v_new=g["in_vn"].copy(), w_new=g["in_wn"].copy(), p=np.zeros(m.n),
             p_rhs=np.zeros(m.n), nu_t=np.zeros(m.n), solid=g["in_solid"])
    oracle_lib.velocity_bcs(m, f["u"], f["v"], f["w"], f["solid"])
    its, dts = [], []
    for step in range(3):
        prm = O.StepParams(nu=nu, rho=rho, cs=0.18, cfl_conv=0.4, cfl_visc=0.2, dt_max=1e-4,
                           solver=kind, pc=pc, max_iter=200 if kind == 0 else (100 if kind == 1 else 40),
                           tol=1e-6, rel_tol=1e-8 if kind == 0 else 0.0, omega=1.7, lmin=lmin,
                           lmax=lmax, degree=4, dt_fixed=(-1.0 if step == 2 else dt))
        it, dto = oracle_lib.step(m, f, A0, A0 if fac == "A" else L0, prm)
        its.append(it)
        dts.append(dto)
    assert list(g["traj%d_dt" % solver]) == dts
    if kind == 0:
        assert its == list(g["traj%d_iters" % solver])
    for k, gk in (("u", "u"), ("v", "v"), ("w", "w"), ("u_new", "un"), ("v_new", "vn"),
                  ("w_new", "wn"), ("p", "p"), ("p_rhs", "p_rhs"), ("nu_t", "nu_t")):
        assert same(f[k], g["traj%d_%s" % (solver, gk)]), k
