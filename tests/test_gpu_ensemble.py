"""Ensembles (one CUDA graph launch per step for many ragged cases) and the
autotuner of the fused inner passes.

In the branch form an ensemble case runs exactly the kernels of the same case
stepped alone through les_step (graph mode), so fields and statistics must be
identical.  In the batched form the cases' solves share kernels and the
column passes march whole-length strips, so the FP32 inner sums round
differently: statistics and fields are held to the mixed-precision bars."""
import numpy as np
import pytest

from conftest import maxrel, same

import les_cases
import les_gb300 as G

pytestmark = pytest.mark.gpu


def _setup(c, spec):
    shape = spec["shape"]
    n = int(np.prod(shape))
    c.upload_mask(np.zeros(n, np.uint8))
    c.build_stencil()          # the reference's order: matrix before the obstacle
    lmax = c.lambda_max(20)
    solid = les_cases.box_mask(shape, spec["box"])
    f = les_cases.init_fields(shape, spec["noise"], spec["seed"])
    les_cases.velocity_bcs_np(shape, f, solid)
    c.upload_fields(f)
    c.upload_mask(solid)
    return lmax


def _params(spec, lmax):
    return G.step_params(nu=les_cases.NU, rho=les_cases.RHO, cs=spec["cs"], cfl_conv=les_cases.CFL_CONV,
                         solver=G.SOLVER_PCG, rel_tol=1e-8,
                         pcg=G.pcg_opts(precond=G.PC_CHEBYSHEV, max_iter=5000, lambda_min=3 * np.pi ** 2,
                                        lambda_max=lmax, degree=4, precision=G.MIXED, inner_rtol=1e-4))


def _specs(count, seed):
    specs = les_cases.batch_cases(count, seed)
    for s in specs:   # keep the test quick: the two smallest extents of the ensemble's range
        s["shape"] = tuple(min(d, 48) for d in s["shape"])
        side = min(s["shape"]) // 4
        s["box"] = (2, 2 + side, 2, 2 + side, 3, 3 + side)
    return specs


def _mesh(spec):
    h = spec["h"]
    return G.Mesh(*spec["shape"], h, h, h)


def _alone(spec, steps):
    with G.Context(_mesh(spec)) as c:
        p = _params(spec, _setup(c, spec))
        st = [c.step(p) for _ in range(steps)]
        return st, c.download_fields()


def test_ensemble_matches_cases_stepped_alone():
    specs = _specs(5, 11)
    steps = 3
    with G.Ensemble([_mesh(s) for s in specs]) as ens:
        ens.set_batched(0)
        prm = [_params(s, _setup(c, s)) for c, s in zip(ens.cases, specs)]
        est = [ens.step(prm) for _ in range(steps)]
        efields = [c.download_fields() for c in ens.cases]
    for i, s in enumerate(specs):
        with G.Context(_mesh(s)) as c:
            p = _params(s, _setup(c, s))
            for k in range(steps):
                st = c.step(p)
                e = est[k][i]
                assert (st.dt, st.iters, st.outer, st.residual, st.status) == \
                       (e.dt, e.iters, e.outer, e.residual, e.status), (i, k)
                assert st.status == G.OK and st.residual < 1e-8 * st.b_norm
            f = c.download_fields()
        for key in ("u", "v", "w", "p", "nu_t", "p_rhs"):
            assert same(f[key], efields[i][key]), (i, key)


@pytest.mark.parametrize("batched", [1, 0], ids=["batched", "branches"])
def test_ensemble_autotune_keeps_the_solution(batched):
    """The ensemble autotuner -- the batched form's work split (timed
    batched iterations over all cases, frozen states), or each case's strip
    shape for the branch form -- changes how the work is cut, not the
    solution; the step after it starts from a fresh solver state."""
    specs = _specs(4, 23)
    with G.Ensemble([_mesh(s) for s in specs]) as ens:
        ens.set_batched(batched)
        prm = [_params(s, _setup(c, s)) for c, s in zip(ens.cases, specs)]
        us = ens.autotune(prm[0].pcg)
        assert us > 0
        if batched:
            assert ens.batch_split() in (2, 3, 4, 6)
        stats = ens.step(prm)
        tuned = [c.download("p") for c in ens.cases]
    for i, s in enumerate(specs):
        assert stats[i].status == G.OK and stats[i].residual < 1e-8 * stats[i].b_norm
        with G.Context(_mesh(s)) as c:
            p = _params(s, _setup(c, s))
            c.step(p)
            # another strip shape rounds the FP32 inner sums differently; the
            # outer FP64 correction holds both to the mixed-vs-FP64 bar
            assert maxrel(c.download("p"), tuned[i]) < 1e-6


def test_autotune_single_context():
    """The autotuner times whole inner iterations (pass A then pass B) and
    leaves its choice in the strip-shape options, where les_get_option reads
    it back: rows of pass A 8 or 16, of pass B 4 or 8 (Chebyshev degree 4),
    chunk lengths within the grid; the step then converges with it."""
    spec = dict(shape=(96, 48, 64), h=1.0 / 32, box=(20, 32, 10, 22, 20, 32), cs=0.17, seed=3, noise=0.01)
    with G.Context(_mesh(spec)) as c:
        p = _params(spec, _setup(c, spec))
        us = c.autotune(p.pcg)
        assert 0 < us < 1e5
        assert c.get_option(G.OPT_ROWS_A) in (8, 16) and c.get_option(G.OPT_ROWS_B) in (4, 8)
        assert 1 <= c.get_option(G.OPT_CHUNK_A) <= 96 and 1 <= c.get_option(G.OPT_CHUNK_B) <= 96
        st = c.step(p)
        assert st.status == G.OK and st.residual < 1e-8 * st.b_norm


def test_options_read_back():
    """les_get_option returns each option's default, then the value set."""
    spec = dict(shape=(24, 12, 12), h=1.0 / 32, box=(8, 12, 4, 8, 4, 8), cs=0.17, seed=1, noise=0.01)
    with G.Context(_mesh(spec)) as c:
        defaults = {G.OPT_FUSED: 1, G.OPT_TMA: 0, G.OPT_ROWS_A: 0, G.OPT_ROWS_B: 0, G.OPT_CHUNK_A: 0,
                    G.OPT_CHUNK_B: 0, G.OPT_GRAPH: 1, G.OPT_PDL: 1, G.OPT_PHYS32: 1, G.OPT_TEST_STALL: 0,
                    G.OPT_COL_STRIDE: 1}
        for opt, v in defaults.items():
            assert c.get_option(opt) == v, (opt, c.get_option(opt), v)
        for opt, v in ((G.OPT_FUSED, 2), (G.OPT_ROWS_A, 16), (G.OPT_CHUNK_B, 12), (G.OPT_GRAPH, 0),
                       (G.OPT_COL_STRIDE, 0)):
            c.set_option(opt, v)
            assert c.get_option(opt) == v
        with pytest.raises(Exception):
            c.get_option(99)


@pytest.mark.parametrize("count,seed", [(6, 5), (3, 17)])
def test_batched_ensemble_close_to_cases_stepped_alone(count, seed):
    """All cases' solves in shared kernels (the default form): every case
    converges to the same relative residual with about the same work as when
    stepped alone, and its fields agree to the mixed-precision bars, over
    steps where the cases finish their solves at different iterations."""
    specs = _specs(count, seed)
    steps = 3
    with G.Ensemble([_mesh(s) for s in specs]) as ens:
        prm = [_params(s, _setup(c, s)) for c, s in zip(ens.cases, specs)]
        est = [ens.step(prm) for _ in range(steps)]
        efields = [c.download_fields() for c in ens.cases]
        launches = sum(c.launch_count() for c in ens.cases)
    assert launches > 0
    for i, s in enumerate(specs):
        alone, f = _alone(s, steps)
        for k in range(steps):
            a, e = alone[k], est[k][i]
            assert e.status == G.OK and e.residual < 1e-8 * e.b_norm, (i, k, e.residual, e.b_norm)
            assert a.dt == e.dt, (i, k)
            assert abs(a.iters - e.iters) <= max(3, 0.15 * a.iters), (i, k, a.iters, e.iters)
        for key, bar in (("u", 1e-7), ("v", 1e-7), ("w", 1e-7), ("p", 1e-6), ("nu_t", 1e-5)):
            assert maxrel(f[key], efields[i][key]) < bar, (i, key, maxrel(f[key], efields[i][key]))


def test_batched_and_branch_forms_switch():
    """Switching the form recaptures the step graph; a mix of preconditioners
    cannot batch and runs as branches."""
    specs = _specs(3, 29)
    with G.Ensemble([_mesh(s) for s in specs]) as ens:
        prm = [_params(s, _setup(c, s)) for c, s in zip(ens.cases, specs)]
        ens.step(prm)
        ens.set_batched(0)
        ens.step(prm)
        ens.set_batched(1)
        prm[1].pcg.degree = 3   # another Chebyshev degree: not batchable
        st = ens.step(prm)
        for x in st:
            assert x.status == G.OK and x.residual < 1e-8 * x.b_norm


def test_batched_ensemble_case_hitting_its_cap():
    """A case whose iteration cap is too small ends NOT_CONVERGED after its
    cap while the other cases of the shared loops converge (the loops run
    while any case iterates, and every pass advances each unfinished case)."""
    specs = _specs(3, 41)
    with G.Ensemble([_mesh(s) for s in specs]) as ens:
        prm = [_params(s, _setup(c, s)) for c, s in zip(ens.cases, specs)]
        prm[1].pcg.max_iter = 30            # total inner iterations of the solve
        prm[1].pcg.inner_max_iter = 30
        st = ens.step(prm)
    assert st[1].status == G.NOT_CONVERGED and st[1].iters <= 31, (st[1].status, st[1].iters)
    for i in (0, 2):
        assert st[i].status == G.OK and st[i].residual < 1e-8 * st[i].b_norm, (i, st[i].status)
