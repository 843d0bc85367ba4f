"""Generates the golden fixtures in tests/golden/*.npz from the compiled
les-model reference (oracle/_ref/libles_ref.so, built by oracle/build_ref.sh
from the reference sources).

The reference ships no numeric fixtures (its only test is a checkpoint round
trip), so these vectors are the pin for the oracle and the CUDA path: every
output below is produced by the reference's own functions, run with one
OpenMP thread so that reductions are plain left-to-right sums.

Run where a les-model checkout exists, with REF naming it:
    REF=<checkout> python tests/golden/make_golden.py
"""
import math
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))

# name, (nx, ny, nz), (dx, dy, dz), mask recipe, seed
GRIDS = [
    ("box12", (12, 10, 9), (1 / 32, 1 / 32, 1 / 32), "box", 11),
    ("aniso16", (16, 8, 8), (0.02, 0.015, 0.01), "random", 12),
    ("tiny7", (7, 5, 3), (0.05, 0.04, 0.03), "random", 13),
]

DT, NU, RHO = 1e-4, 1e-5, 1.2
NOISE = 0.1


def make_mask(shape, recipe, rng):
    nx, ny, nz = shape
    s = np.zeros(shape, np.uint8)
    if recipe == "box":
        s[4:7, 3:6, 3:6] = 1
    else:
        s[:] = (rng.random(shape) < 0.12).astype(np.uint8)
        # always exercise: a solid inlet cell, a solid cell next to the outlet,
        # and a fully enclosed solid cell
        s[0, ny // 2, nz // 2] = 1
        s[nx - 2, 1, 1] = 1
        if min(shape) >= 5:
            c = (nx // 2, ny // 2, nz // 2)
            s[c[0] - 1:c[0] + 2, c[1] - 1:c[1] + 2, c[2] - 1:c[2] + 2] = 1
    return s.reshape(-1)


def run(name, shape, h, recipe, seed, ref):
    rng = np.random.default_rng(seed)
    m = O.Mesh(*shape, *h)
    n = m.n
    d = {}
    solid = make_mask(shape, recipe, rng)
    u = 1.0 + rng.uniform(-NOISE, NOISE, n)
    v = rng.uniform(-NOISE, NOISE, n)
    w = rng.uniform(-NOISE, NOISE, n)
    un, vn, wn = (rng.uniform(-NOISE, NOISE, n) for _ in range(3))
    un += 1.0
    p = rng.uniform(-1.0, 1.0, n)
    nu_t = rng.uniform(0.0, 1e-4, n)
    r = rng.uniform(-1.0, 1.0, n)
    for k, a in dict(solid=solid, u=u, v=v, w=w, un=un, vn=vn, wn=wn, p=p, nu_t=nu_t, r=r).items():
        d["in_" + k] = a.copy()
    d["mesh"] = np.array([*shape], np.int64)
    d["h"] = np.array(h, np.float64)
    d["scal"] = np.array([DT, NU, RHO], np.float64)

    # --- step physics (src/main.cpp)
    a = [x.copy() for x in (u, v, w)]
    ref.velocity_bcs(m, *a, solid)
    d["out_vbc_u"], d["out_vbc_v"], d["out_vbc_w"] = a

    nt = nu_t.copy()
    tau = np.zeros(6 * n)
    ref.sgs(m, u, v, w, nt, tau)
    d["out_sgs_nu_t"], d["out_sgs_tau"] = nt, tau

    nt2 = nt.copy()
    ref.nut_bcs(m, nt2, solid)
    d["out_nutbc_nu_t"] = nt2

    outs = [np.zeros(n) for _ in range(6)]
    ref.momentum(m, DT, NU, u, v, w, un, vn, wn, nt2, *outs)
    for k, a in zip(("u", "v", "w", "un", "vn", "wn"), outs):
        d["out_mom_" + k] = a

    a = [x.copy() for x in (u, v, w)]
    ref.correct_velocity(m, DT, RHO, p, *a)
    d["out_corr_u"], d["out_corr_v"], d["out_corr_w"] = a

    d["out_dt"] = np.array([ref.adaptive_dt(m, u, v, w, nu_t, NU)])

    # --- pressure (src/pressure.cpp)
    pp = p.copy()
    ref.pressure_bcs(m, pp, solid)
    d["out_pbc_p"] = pp

    pp = p.copy()
    ref.solve_jacobi(m, DT, RHO, u, v, w, pp, solid)
    d["out_jac_p"] = pp
    pp = p.copy()
    ref.solve_gs(m, DT, RHO, u, v, w, pp, solid, 30)
    d["out_gs_p"] = pp

    div = np.zeros(n)
    ref.divergence(m, DT, RHO, un, vn, wn, solid, div)
    d["out_div"] = div
    b = np.zeros(n)
    ref.build_b(m, div, solid, b)
    d["out_b"] = b

    for tag, msk in (("", solid), ("0", np.zeros(n, np.uint8))):
        A = O.new_stencil(n)
        ref.build_stencil(m, msk, A)
        for k in O.DIAGS:
            d["out_A%s_%s" % (tag, k)] = A[k]
    A = {k: d["out_A_" + k] for k in O.DIAGS}
    A0 = {k: d["out_A0_" + k] for k in O.DIAGS}

    q = np.zeros(n)
    ref.spmv(m, A, p, q)
    d["out_spmv_q"] = q
    z = np.zeros(n)
    ref.jacobi_precond(m, A, r, z)
    d["out_jpc_z"] = z

    Lm = O.new_stencil(n)
    ref.ic_build(m, A, Lm)
    for k in O.DIAGS:
        d["out_L_" + k] = Lm[k]
    L0 = O.new_stencil(n)
    ref.ic_build(m, A0, L0)
    for k in O.DIAGS:
        d["out_L0_" + k] = L0[k]
    z = np.zeros(n)
    ref.ic_apply(m, Lm, r, z)
    d["out_icL_z"] = z
    z = np.zeros(n)
    ref.ic_apply(m, A, r, z)
    d["out_icA_z"] = z

    lmax = ref.lambda_max(m, A0, 20)
    lmin = 3.0 * math.pi ** 2
    d["out_lmax"] = np.array([lmax, lmin])
    z = np.zeros(n)
    ref.cheb_apply(m, A0, lmin, lmax, 4, r, z)
    d["out_cheb_z"] = z

    # --- PCG solves on the system of src/main.cpp's build order (A from the
    # empty mask), b from the divergence above, x0 = p
    tol = 1e-8 * np.linalg.norm(b)
    d["pcg_tol"] = np.array([tol])
    its = []
    x = p.copy(); its.append(ref.pcg_shipped(m, A0, b, x, 60, tol)); d["out_pcg_shipped_x"] = x
    x = p.copy(); its.append(ref.pcg_cheb(m, A0, b, x, lmin, lmax, 4, 300, tol)); d["out_pcg_cheb_x"] = x
    x = p.copy(); its.append(ref.pcg_restated(m, A0, None, 0, b, x, 300, tol)); d["out_pcg_jac_x"] = x
    x = p.copy(); its.append(ref.pcg_restated(m, A0, L0, 1, b, x, 300, tol)); d["out_pcg_icL_x"] = x
    d["out_pcg_iters"] = np.array(its, np.int64)

    # --- short trajectories through the full step (src/main.cpp:108-165)
    import ctypes as C
    for solver in range(6):
        f = dict(u=u.copy(), v=v.copy(), w=w.copy(), un=un.copy(), vn=vn.copy(), wn=wn.copy(),
                 p=np.zeros(n), p_rhs=np.zeros(n), nu_t=np.zeros(n))
        ref.velocity_bcs(m, f["u"], f["v"], f["w"], solid)
        its, dts = [], []
        for step in range(3):
            dto = C.c_double(0)
            it = ref.step(m, f["u"], f["v"], f["w"], f["un"], f["vn"], f["wn"], f["p"], f["p_rhs"],
                          f["nu_t"], solid, A0, L0, solver, -1.0 if step == 2 else DT, NU, RHO, 200,
                          1e-8, lmin, lmax, 4, 40, C.byref(dto))
            its.append(it)
            dts.append(dto.value)
        for k in ("u", "v", "w", "un", "vn", "wn", "p", "p_rhs", "nu_t"):
            d["traj%d_%s" % (solver, k)] = f[k]
        d["traj%d_iters" % solver] = np.array(its, np.int64)
        d["traj%d_dt" % solver] = np.array(dts)

    np.savez_compressed(os.path.join(OUT, name + ".npz"), **d)
    print(name, "pcg iters", d["out_pcg_iters"], "lmax %.6f" % lmax,
          "traj iters", [list(d["traj%d_iters" % s]) for s in range(6)])


def run_io(ref):
    """Statistics (src/statistics.cpp) and file formats (src/io.cpp) on a
    7x5x3 grid: three sampled steps with start_step 0 (the reference skips
    step 0), the ten sums, the statistics file, one field file and one
    checkpoint, stored as bytes."""
    import ctypes as C
    import tempfile
    shape, h = (7, 5, 3), (0.125, 0.2, 1.0 / 3)
    m = O.Mesh(*shape, *h)
    n = m.n
    rng = np.random.default_rng(77)
    steps = [[rng.standard_normal(n) * s for s in (1.0, 0.3, 0.2, 2.0)] for _ in range(3)]
    sums = [np.zeros(n) for _ in range(10)]
    keep = [a for st in steps for a in st]
    arr = (C.POINTER(C.c_double) * 12)(*[O._p(a) for a in keep])
    outs = (C.POINTER(C.c_double) * 10)(*[O._p(a) for a in sums])
    d = {}
    with tempfile.TemporaryDirectory() as tmp:
        os.makedirs(os.path.join(tmp, "output"))
        os.makedirs(os.path.join(tmp, "checkpoint"))
        ns = ref.lib.ref_statistics(*ref._m(m), 3, 0, arr, outs, tmp.encode(), b"stats.vtk")
        d["stats_samples"] = np.array([ns])
        for s, st in enumerate(steps):
            for k, a in zip(("u", "v", "w", "p"), st):
                d["stats_in%d_%s" % (s, k)] = a
        for q, k in enumerate(("u", "v", "w", "p", "uu", "vv", "ww", "uv", "uw", "vw")):
            d["stats_sum_" + k] = sums[q]
        d["stats_vtk"] = np.frombuffer(open(os.path.join(tmp, "stats.vtk"), "rb").read(), np.uint8)
        f = {k: rng.standard_normal(n) for k in ("u", "v", "w", "p")}
        f["nu_t"] = np.abs(rng.standard_normal(n)) * 1e-3
        f["u"][3] = 1.0 / 3.0          # a few values that exercise %g rounding and exponents
        f["v"][4] = -2.5e-7
        f["p"][5] = 123456789.0
        solid = (rng.random(n) < 0.3).astype(np.uint8)
        for k, v in f.items():
            d["io_" + k] = v
        d["io_solid"] = solid
        ref.lib.ref_write_field_vtk(*ref._m(m), *[O._p(f[k]) for k in ("u", "v", "w", "p", "nu_t")],
                                    solid.ctypes.data_as(C.POINTER(C.c_uint8)), C.c_int(42), tmp.encode())
        d["io_vtk_step"] = np.array([42])
        d["io_vtk"] = np.frombuffer(open(os.path.join(tmp, "output", "output_42.vtk"), "rb").read(), np.uint8)
        t_sim, dt, nxt = 0.0123456789012345678, 1e-4 / 3.0, 17
        ref.lib.ref_save_state(*ref._m(m), *[O._p(f[k]) for k in ("u", "v", "w", "p", "nu_t")],
                               solid.ctypes.data_as(C.POINTER(C.c_uint8)), C.c_double(t_sim), C.c_double(dt),
                               C.c_int(nxt), tmp.encode())
        d["ckpt_args"] = np.array([t_sim, dt, nxt])
        d["ckpt_meta"] = np.frombuffer(open(os.path.join(tmp, "checkpoint", "checkpoint.meta"), "rb").read(), np.uint8)
        d["ckpt_data"] = np.frombuffer(open(os.path.join(tmp, "checkpoint", "checkpoint.data"), "rb").read(), np.uint8)
    d["mesh"] = np.array([*shape, *h])
    np.savez_compressed(os.path.join(OUT, "io_tiny7.npz"), **d)
    print("io_tiny7: samples", ns, "stats file", d["stats_vtk"].size, "B, field file", d["io_vtk"].size,
          "B, checkpoint", d["ckpt_meta"].size, "+", d["ckpt_data"].size, "B")


def main():
    O.build_ref()
    ref = O.Ref()
    ref.set_threads(1)
    for g in GRIDS:
        run(*g, ref)
    run_io(ref)


if __name__ == "__main__":
    main()
