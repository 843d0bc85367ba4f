"""ctypes binding of the les_gb300 C ABI (include/les_gb300.h).

This is how the tests and bench.py drive the CUDA library: every call goes
through the same extern "C" entry points a C/C++ host (or the reference-API
shim) would use.  There is no fallback: if libles_gb300.so is missing or no
GPU is present the calls raise.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
LIB_PATH = os.path.join(PKG, "libles_gb300.so")

# status codes
OK, NOT_CONVERGED, NONFINITE, BAD_ARG, CUDA_ERROR, NO_DEVICE, TIMEOUT = range(7)
# slots
U, V, W, U_NEW, V_NEW, W_NEW, P, P_RHS, NU_T, B = range(10)
SLOTS = {"u": U, "v": V, "w": W, "u_new": U_NEW, "v_new": V_NEW, "w_new": W_NEW, "p": P,
         "p_rhs": P_RHS, "nu_t": NU_T, "b": B}
# solvers, preconditioners, precision
SOLVER_PCG, SOLVER_JACOBI, SOLVER_GS = 0, 1, 2
PC_JACOBI, PC_IC, PC_CHEBYSHEV, PC_IC_A = 0, 1, 2, 3
FP64, MIXED = 0, 1
(OPT_FUSED, OPT_TMA, OPT_ROWS_A, OPT_ROWS_B, OPT_CHUNK_A, OPT_CHUNK_B, OPT_GRAPH, OPT_PDL, OPT_PHYS32,
 OPT_TEST_STALL, OPT_COL_STRIDE) = range(11)
DIAGS = ("c", "n", "s", "e", "w", "t", "b")

_dp = C.POINTER(C.c_double)
_u8 = C.POINTER(C.c_uint8)


class LesError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("les_gb300 status %d: %s" % (status, msg))
        self.status = status


class Mesh(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double)]

    @property
    def n(self):
        return self.nx * self.ny * self.nz


class PcgOpts(C.Structure):
    _fields_ = [("precond", C.c_int), ("max_iter", C.c_int), ("tol", C.c_double),
                ("lambda_min", C.c_double), ("lambda_max", C.c_double), ("degree", C.c_int),
                ("precision", C.c_int), ("inner_rtol", C.c_double), ("inner_max_iter", C.c_int),
                ("max_outer", C.c_int)]


class PcgResult(C.Structure):
    _fields_ = [("iters", C.c_int), ("outer", C.c_int), ("residual", C.c_double)]


class StepParams(C.Structure):
    _fields_ = [("nu", C.c_double), ("rho", C.c_double), ("cs", C.c_double),
                ("cfl_conv", C.c_double), ("cfl_visc", C.c_double), ("dt_max", C.c_double),
                ("dt_fixed", C.c_double), ("solver", C.c_int), ("pcg", PcgOpts),
                ("rel_tol", C.c_double), ("stat_max_iter", C.c_int), ("stat_tol", C.c_double),
                ("omega", C.c_double), ("want_tau", C.c_int)]


class AdjointParams(C.Structure):
    _fields_ = [("step", StepParams), ("steps", C.c_int), ("checkpoint_every", C.c_int),
                ("box", C.c_int * 6), ("adj_rel_tol", C.c_double)]


class StepStats(C.Structure):
    _fields_ = [("dt", C.c_double), ("iters", C.c_int), ("outer", C.c_int),
                ("residual", C.c_double), ("b_norm", C.c_double), ("status", C.c_int)]


def pcg_opts(precond=PC_JACOBI, max_iter=1000, tol=1e-6, lambda_min=0.0, lambda_max=0.0, degree=5,
             precision=FP64, inner_rtol=1e-4, inner_max_iter=0, max_outer=50):
    return PcgOpts(precond, max_iter, tol, lambda_min, lambda_max, degree, precision, inner_rtol,
                   inner_max_iter, max_outer)


def step_params(**kw):
    """Reference defaults (src/main.cpp:83-87, :137, :210-212, :425;
    src/pressure.cpp:134, :195)."""
    d = dict(nu=1e-5, rho=1.2, cs=0.18, cfl_conv=0.4, cfl_visc=0.2, dt_max=1e-4, dt_fixed=0.0,
             solver=SOLVER_PCG, rel_tol=0.0, stat_max_iter=100, stat_tol=1e-6, omega=1.7, want_tau=0)
    pcg = kw.pop("pcg", None) or pcg_opts(precond=PC_IC_A, max_iter=1000, tol=1e-6)
    d.update(kw)
    return StepParams(d["nu"], d["rho"], d["cs"], d["cfl_conv"], d["cfl_visc"], d["dt_max"],
                      d["dt_fixed"], d["solver"], pcg, d["rel_tol"], d["stat_max_iter"], d["stat_tol"],
                      d["omega"], d["want_tau"])


_lib = None


def load(path=None):
    """Loads libles_gb300.so; raises if it has not been built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise FileNotFoundError("%s is missing: run les-model_gb300/build_ext.py (or "
                                "__graft_entry__.build())" % p)
    L = C.CDLL(p)
    L.les_last_error.restype = C.c_char_p
    L.les_status_string.restype = C.c_char_p
    L.les_stream.restype = C.c_void_p
    L.les_slot_ptr.restype = C.c_void_p
    L.les_mask_ptr.restype = C.c_void_p
    L.les_create.argtypes = [C.POINTER(Mesh), C.c_int, C.POINTER(C.c_void_p)]
    L.les_destroy.argtypes = [C.c_void_p]
    for name in ("les_last_error", "les_sync", "les_stream", "les_velocity_bcs", "les_nut_bcs",
                 "les_build_b", "les_pressure_bcs", "les_build_stencil", "les_build_ic"):
        getattr(L, name).argtypes = [C.c_void_p]
    if path is None:
        _lib = L
    return L


def exported_symbols():
    """Names the header declares (parsed from include/les_gb300.h)."""
    import re
    hdr = os.path.join(os.path.dirname(PKG), "include", "les_gb300.h")
    src = open(hdr).read()
    return sorted(set(re.findall(r"^\s*(?:[A-Za-z_][\w\s\*]*?)\b(les_\w+)\s*\(", src, re.M)))


def _arr(a, dtype=np.float64):
    a = np.ascontiguousarray(a, dtype=dtype)
    return a


class Context:
    """One device context (a Field mirror + pressure system on one GPU)."""

    def __init__(self, mesh, device=0, lib=None):
        self.lib = lib or load()
        self.mesh = mesh
        self.n = mesh.n
        h = C.c_void_p()
        st = self.lib.les_create(C.byref(mesh), device, C.byref(h))
        if st != OK:
            raise LesError(st, self.lib.les_status_string(st).decode())
        self.h = h

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _chk(self, st, allow=(OK,)):
        if st not in allow:
            raise LesError(st, self.lib.les_last_error(self.h).decode())
        return st

    # --- plumbing
    @property
    def stream(self):
        return self.lib.les_stream(self.h)

    def slot_ptr(self, slot):
        return self.lib.les_slot_ptr(self.h, SLOTS.get(slot, slot))

    def sync(self):
        self._chk(self.lib.les_sync(self.h))

    def upload(self, slot, a):
        a = _arr(a)
        assert a.size == self.n
        self._chk(self.lib.les_upload(self.h, SLOTS.get(slot, slot), a.ctypes.data_as(_dp)))

    def upload_ptr(self, slot, ptr):
        self._chk(self.lib.les_upload(self.h, SLOTS.get(slot, slot), C.cast(ptr, _dp)))

    def download(self, slot, out=None):
        out = np.empty(self.n) if out is None else out
        self._chk(self.lib.les_download(self.h, SLOTS.get(slot, slot), out.ctypes.data_as(_dp)))
        return out

    def download_ptr(self, slot, ptr):
        self._chk(self.lib.les_download(self.h, SLOTS.get(slot, slot), C.cast(ptr, _dp)))

    def upload_many_ptr(self, slot_ptrs):
        """{slot: host pointer} in one call (one synchronisation)."""
        n = len(slot_ptrs)
        sl = (C.c_int * n)(*[SLOTS.get(k, k) for k in slot_ptrs])
        ps = (_dp * n)(*[C.cast(p, _dp) for p in slot_ptrs.values()])
        self._chk(self.lib.les_upload_many(self.h, n, sl, ps))

    def download_many_ptr(self, slot_ptrs):
        n = len(slot_ptrs)
        sl = (C.c_int * n)(*[SLOTS.get(k, k) for k in slot_ptrs])
        ps = (_dp * n)(*[C.cast(p, _dp) for p in slot_ptrs.values()])
        self._chk(self.lib.les_download_many(self.h, n, sl, ps))

    def upload_mask(self, m):
        m = _arr(m, np.uint8)
        assert m.size == self.n
        self._chk(self.lib.les_upload_mask(self.h, m.ctypes.data_as(_u8)))

    def download_mask(self):
        out = np.empty(self.n, np.uint8)
        self._chk(self.lib.les_download_mask(self.h, out.ctypes.data_as(_u8)))
        return out

    def upload_fields(self, f):
        for k, v in f.items():
            if k == "solid":
                self.upload_mask(v)
            elif k in SLOTS:
                self.upload(k, v)

    def download_fields(self, keys=("u", "v", "w", "u_new", "v_new", "w_new", "p", "p_rhs", "nu_t")):
        return {k: self.download(k) for k in keys}

    # --- step physics
    def adaptive_dt(self, nu, cfl_conv=0.4, cfl_visc=0.2, dt_max=1e-4):
        dt = C.c_double()
        self._chk(self.lib.les_adaptive_dt(self.h, C.c_double(nu), C.c_double(cfl_conv),
                                           C.c_double(cfl_visc), C.c_double(dt_max), C.byref(dt)))
        return dt.value

    def velocity_bcs(self):
        self._chk(self.lib.les_velocity_bcs(self.h))

    def sgs(self, cs, want_tau=False):
        self._chk(self.lib.les_sgs(self.h, C.c_double(cs), int(want_tau)))

    def nut_bcs(self):
        self._chk(self.lib.les_nut_bcs(self.h))

    def sgs_nut(self, cs, want_tau=False):
        self._chk(self.lib.les_sgs_nut(self.h, C.c_double(cs), int(want_tau)))

    def download_tau(self):
        out = np.empty(6 * self.n)
        self._chk(self.lib.les_download_tau(self.h, out.ctypes.data_as(_dp)))
        return out

    def momentum(self, dt, nu):
        self._chk(self.lib.les_momentum(self.h, C.c_double(dt), C.c_double(nu)))

    def correct_velocity(self, dt, rho):
        self._chk(self.lib.les_correct_velocity(self.h, C.c_double(dt), C.c_double(rho)))

    # --- pressure
    def divergence(self, dt, rho):
        self._chk(self.lib.les_divergence(self.h, C.c_double(dt), C.c_double(rho)))

    def build_b(self):
        self._chk(self.lib.les_build_b(self.h))

    def pressure_bcs(self):
        self._chk(self.lib.les_pressure_bcs(self.h))

    def solve_jacobi(self, dt, rho, max_iter=100, tol=1e-6):
        it = C.c_int()
        self._chk(self.lib.les_solve_jacobi(self.h, C.c_double(dt), C.c_double(rho), int(max_iter),
                                            C.c_double(tol), C.byref(it)))
        return it.value

    def solve_gs(self, dt, rho, max_iter=200, omega=1.7, tol=1e-6):
        it = C.c_int()
        self._chk(self.lib.les_solve_gs(self.h, C.c_double(dt), C.c_double(rho), int(max_iter),
                                        C.c_double(omega), C.c_double(tol), C.byref(it)))
        return it.value

    def build_stencil(self):
        self._chk(self.lib.les_build_stencil(self.h))

    def _d7(self, d):
        arrs = [_arr(d[k]) for k in DIAGS]
        ptrs = (_dp * 7)(*[a.ctypes.data_as(_dp) for a in arrs])
        return ptrs, arrs

    def set_stencil(self, d):
        ptrs, keep = self._d7(d)
        self._chk(self.lib.les_set_stencil(self.h, ptrs))

    def get_stencil(self):
        d = {k: np.empty(self.n) for k in DIAGS}
        ptrs, _ = self._d7(d)
        self._chk(self.lib.les_get_stencil(self.h, ptrs))
        return d

    def build_ic(self):
        self._chk(self.lib.les_build_ic(self.h))

    def set_ic_factor(self, d):
        ptrs, keep = self._d7(d)
        self._chk(self.lib.les_set_ic_factor(self.h, ptrs))

    def get_ic_factor(self):
        d = {k: np.empty(self.n) for k in DIAGS}
        ptrs, _ = self._d7(d)
        self._chk(self.lib.les_get_ic_factor(self.h, ptrs))
        return d

    def lambda_max(self, n_iter=20, v0=None):
        lam = C.c_double()
        if v0 is not None:
            v0 = _arr(v0)
        self._chk(self.lib.les_lambda_max(self.h, int(n_iter),
                                          v0.ctypes.data_as(_dp) if v0 is not None else None,
                                          C.byref(lam)))
        return lam.value

    def pcg(self, opts):
        r = PcgResult()
        st = self.lib.les_pcg(self.h, C.byref(opts), C.byref(r))
        self._chk(st, allow=(OK, NOT_CONVERGED, NONFINITE))
        return st, r

    def spmv(self, src, dst):
        self._chk(self.lib.les_spmv(self.h, SLOTS.get(src, src), SLOTS.get(dst, dst)))

    def precond_apply(self, opts, src, dst):
        self._chk(self.lib.les_precond_apply(self.h, C.byref(opts), SLOTS.get(src, src),
                                             SLOTS.get(dst, dst)))

    def dot(self, a, b):
        out = C.c_double()
        self._chk(self.lib.les_dot(self.h, SLOTS.get(a, a), SLOTS.get(b, b), C.byref(out)))
        return out.value

    def step(self, params):
        s = StepStats()
        self._chk(self.lib.les_step(self.h, C.byref(params), C.byref(s)))
        return s

    def step_io(self, params, up, down):
        """One step with host fields: {slot: host pointer} uploaded before it,
        {slot: host pointer} downloaded after it (les_step_io); returns
        (stats, device ms of the step)."""
        s = StepStats()
        ms = C.c_double()
        ni, no = len(up), len(down)
        si = (C.c_int * max(ni, 1))(*[SLOTS.get(k, k) for k in up])
        pi = (_dp * max(ni, 1))(*[C.cast(p, _dp) for p in up.values()])
        so = (C.c_int * max(no, 1))(*[SLOTS.get(k, k) for k in down])
        po = (_dp * max(no, 1))(*[C.cast(p, _dp) for p in down.values()])
        self._chk(self.lib.les_step_io(self.h, C.byref(params), C.byref(s), ni, si, pi, no, so, po, C.byref(ms)))
        return s, ms.value

    def set_option(self, option, value):
        self._chk(self.lib.les_set_option(self.h, int(option), int(value)))

    def get_option(self, option):
        v = C.c_int()
        self._chk(self.lib.les_get_option(self.h, int(option), C.byref(v)))
        return v.value

    # --- accounting
    def mark(self, slot):
        self._chk(self.lib.les_mark(self.h, int(slot)))

    def elapsed(self, m0, m1):
        ms = C.c_double()
        self._chk(self.lib.les_elapsed(self.h, int(m0), int(m1), C.byref(ms)))
        return ms.value

    def launch_count(self):
        self.lib.les_launch_count.restype = C.c_ulonglong
        self.lib.les_launch_count.argtypes = [C.c_void_p]
        return int(self.lib.les_launch_count(self.h))

    def profile(self, enable):
        self._chk(self.lib.les_profile(self.h, int(enable)))

    def profile_read(self, kernel_id):
        n = C.c_int()
        ms = C.c_double()
        self._chk(self.lib.les_profile_read(self.h, int(kernel_id), C.byref(n), C.byref(ms)))
        return n.value, ms.value

    def profile_all(self):
        self.lib.les_profile_name.restype = C.c_char_p
        out = {}
        for kid in range(8):
            n, ms = self.profile_read(kid)
            if n:
                out[self.lib.les_profile_name(kid).decode()] = (n, ms)
        return out

    def fp64_rate(self):
        """Measured FP64 multiply/add rate of the GPU (operations per second)."""
        r = C.c_double()
        self.lib.les_fp64_rate.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        self._chk(self.lib.les_fp64_rate(self.h, C.byref(r)))
        return r.value

    # --- autotuner
    def autotune(self, opts, share=1.0):
        """Times strip shapes and chunk lengths of the column passes for opts
        and keeps the fastest; returns microseconds per inner iteration."""
        us = C.c_double()
        self.lib.les_autotune.argtypes = [C.c_void_p, C.POINTER(PcgOpts), C.c_double, C.POINTER(C.c_double)]
        self._chk(self.lib.les_autotune(self.h, C.byref(opts), C.c_double(share), C.byref(us)))
        return us.value

    @classmethod
    def borrowed(cls, handle, mesh, lib):
        """A view of a context owned elsewhere (an ensemble case)."""
        self = cls.__new__(cls)
        self.lib, self.mesh, self.n, self.h = lib, mesh, mesh.n, C.c_void_p(handle)
        self._borrowed = True
        return self

    def close(self):
        if self.h and not getattr(self, "_borrowed", False):
            self.lib.les_destroy(self.h)
        self.h = None


class Ensemble:
    """Independent cases advanced by one CUDA graph launch per time step."""

    def __init__(self, meshes, device=0, lib=None):
        self.lib = L = lib or load()
        L.les_ensemble_create.argtypes = [C.POINTER(Mesh), C.c_int, C.c_int, C.POINTER(C.c_void_p)]
        L.les_ensemble_destroy.argtypes = [C.c_void_p]
        L.les_ensemble_case.argtypes = [C.c_void_p, C.c_int]
        L.les_ensemble_case.restype = C.c_void_p
        L.les_ensemble_last_error.argtypes = [C.c_void_p]
        L.les_ensemble_last_error.restype = C.c_char_p
        L.les_ensemble_step.argtypes = [C.c_void_p, C.POINTER(StepParams), C.POINTER(StepStats)]
        L.les_ensemble_sync.argtypes = [C.c_void_p]
        L.les_ensemble_autotune.argtypes = [C.c_void_p, C.POINTER(PcgOpts), C.POINTER(C.c_double)]
        self.n = len(meshes)
        arr = (Mesh * self.n)(*meshes)
        h = C.c_void_p()
        st = L.les_ensemble_create(arr, self.n, device, C.byref(h))
        if st != OK:
            raise LesError(st, L.les_status_string(st).decode())
        self.h = h
        self.cases = [Context.borrowed(L.les_ensemble_case(h, i), meshes[i], L) for i in range(self.n)]

    def _chk(self, st):
        if st != OK:
            raise LesError(st, self.lib.les_ensemble_last_error(self.h).decode())

    def step(self, params, stats=True):
        prm = (StepParams * self.n)(*params)
        if not stats:
            self._chk(self.lib.les_ensemble_step(self.h, prm, None))
            return None
        out = (StepStats * self.n)()
        self._chk(self.lib.les_ensemble_step(self.h, prm, out))
        return list(out)

    def sync(self):
        self._chk(self.lib.les_ensemble_sync(self.h))

    def autotune(self, opts):
        us = C.c_double()
        self._chk(self.lib.les_ensemble_autotune(self.h, C.byref(opts), C.byref(us)))
        return us.value

    def set_batched(self, on):
        """1: the cases' solves run batched (one kernel per pass over all
        cases); 0: one graph branch per case."""
        self._chk(self.lib.les_ensemble_set_batched(self.h, int(on)))

    def batch_split(self):
        """Items of a batched pass, in multiples of the resident warps."""
        return self.lib.les_ensemble_batch_split(self.h)

    def close(self):
        if self.h:
            for c in self.cases:
                c.h = None
            self.lib.les_ensemble_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def _ctx_set_inlet(self, u_in):
    """Inlet u profile (ny*nz, index j*nz+k) or None for the uniform inlet."""
    self.lib.les_set_inlet.argtypes = [C.c_void_p, C.c_void_p]
    if u_in is None:
        self._chk(self.lib.les_set_inlet(self.h, None))
    else:
        a = _arr(u_in)
        assert a.size == self.mesh.ny * self.mesh.nz
        self._chk(self.lib.les_set_inlet(self.h, a.ctypes.data))


def _ctx_adjoint_forward(self, step, steps, checkpoint_every, box, adj_rel_tol=1e-12):
    p = AdjointParams(step, steps, checkpoint_every, (C.c_int * 6)(*box), adj_rel_tol)
    J = C.c_double()
    self.lib.les_adjoint_forward.argtypes = [C.c_void_p, C.POINTER(AdjointParams), C.POINTER(C.c_double)]
    self._chk(self.lib.les_adjoint_forward(self.h, C.byref(p), C.byref(J)))
    return J.value


def _ctx_adjoint_backward(self):
    g = np.zeros(self.mesh.ny * self.mesh.nz)
    gcs = C.c_double()
    self.lib.les_adjoint_backward.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(C.c_double)]
    self._chk(self.lib.les_adjoint_backward(self.h, g.ctypes.data, C.byref(gcs)))
    return g, gcs.value


Context.set_inlet = _ctx_set_inlet
Context.adjoint_forward = _ctx_adjoint_forward
Context.adjoint_backward = _ctx_adjoint_backward


# ---- statistics and files (src/statistics.cpp, src/io.cpp)
_STAT_KEYS = ("u", "v", "w", "p", "uu", "vv", "ww", "uv", "uw", "vw")


def _ptr_array(arrs):
    return (C.POINTER(C.c_double) * len(arrs))(*[None if a is None else a.ctypes.data_as(_dp) for a in arrs])


def _ctx_stats_begin(self, start_step):
    self._chk(self.lib.les_stats_begin(self.h, int(start_step)))


def _ctx_stats_update(self, step):
    self._chk(self.lib.les_stats_update(self.h, int(step)))


def _ctx_stats_read(self, finalize=False):
    out = [np.empty(self.n) for _ in range(10)]
    ns = C.c_int()
    fn = self.lib.les_stats_finalize if finalize else self.lib.les_stats_sums
    self._chk(fn(self.h, _ptr_array(out), C.byref(ns)))
    return dict(zip(_STAT_KEYS, out)), ns.value


def _ctx_stats_save_vtk(self, path):
    self._chk(self.lib.les_stats_save_vtk(self.h, str(path).encode()))


def _ctx_write_vtk(self, step, path):
    self._chk(self.lib.les_write_vtk(self.h, int(step), str(path).encode()))


def _ctx_save_state(self, d, time_simulated, dt, next_step, with_unew=False):
    self._chk(self.lib.les_save_state(self.h, str(d).encode(), C.c_double(time_simulated), C.c_double(dt),
                                      int(next_step), int(with_unew)))


def _ctx_io_wait(self):
    self._chk(self.lib.les_io_wait(self.h))


def _ctx_load_state(self, d, with_unew=False):
    t, dt, step = C.c_double(), C.c_double(), C.c_int()
    self._chk(self.lib.les_load_state(self.h, str(d).encode(), C.byref(t), C.byref(dt), C.byref(step),
                                      int(with_unew)))
    return step.value, t.value, dt.value


Context.stats_begin = _ctx_stats_begin
Context.stats_update = _ctx_stats_update
Context.stats_read = _ctx_stats_read
Context.stats_save_vtk = _ctx_stats_save_vtk
Context.write_vtk = _ctx_write_vtk
Context.save_state = _ctx_save_state
Context.io_wait = _ctx_io_wait
Context.load_state = _ctx_load_state


def format_field_vtk(mesh, step, f, solid, path, lib=None):
    """write_field_vtk from host arrays (no device)."""
    L = lib or load()
    a = [_arr(f[k]) for k in ("u", "v", "w", "p", "nu_t")]
    s = _arr(solid, np.uint8)
    st = L.les_format_field_vtk(C.byref(mesh), int(step), *[x.ctypes.data_as(_dp) for x in a],
                                s.ctypes.data_as(_u8), str(path).encode())
    if st != OK:
        raise LesError(st, "format_field_vtk")


def format_stats_vtk(mesh, mean4, stress6, path, lib=None):
    L = lib or load()
    m4 = [_arr(x) for x in mean4]
    s6 = [_arr(x) for x in stress6]
    st = L.les_format_stats_vtk(C.byref(mesh), _ptr_array(m4), _ptr_array(s6), str(path).encode())
    if st != OK:
        raise LesError(st, "format_stats_vtk")


def write_checkpoint_files(mesh, f, solid, time_simulated, dt, next_step, d, unew3=None, lib=None):
    L = lib or load()
    a = [_arr(f[k]) for k in ("u", "v", "w", "p", "nu_t")]
    s = _arr(solid, np.uint8)
    u3 = [_arr(x) for x in unew3] if unew3 is not None else None
    st = L.les_write_checkpoint_files(C.byref(mesh), _ptr_array(a), s.ctypes.data_as(_u8), C.c_double(time_simulated),
                                      C.c_double(dt), int(next_step), str(d).encode(),
                                      _ptr_array(u3) if u3 is not None else None)
    if st != OK:
        raise LesError(st, "write_checkpoint_files")


def read_checkpoint_files(mesh, d, with_unew=False, lib=None):
    L = lib or load()
    n = mesh.n
    a = [np.empty(n) for _ in range(5)]
    s = np.empty(n, np.uint8)
    u3 = [np.empty(n) for _ in range(3)] if with_unew else None
    t, dt, step = C.c_double(), C.c_double(), C.c_int()
    st = L.les_read_checkpoint_files(C.byref(mesh), str(d).encode(), _ptr_array(a), s.ctypes.data_as(_u8), C.byref(t),
                                     C.byref(dt), C.byref(step), _ptr_array(u3) if u3 is not None else None)
    if st != OK:
        raise LesError(st, "read_checkpoint_files")
    f = dict(zip(("u", "v", "w", "p", "nu_t"), a))
    return step.value, t.value, dt.value, f, s, u3


def _ctx_adjoint_tangent(self, d_inlet, d_cs):
    dJ = C.c_double()
    self.lib.les_adjoint_tangent.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.POINTER(C.c_double)]
    a = None if d_inlet is None else _arr(d_inlet)
    self._chk(self.lib.les_adjoint_tangent(self.h, None if a is None else a.ctypes.data, C.c_double(d_cs),
                                           C.byref(dJ)))
    return dJ.value


Context.adjoint_tangent = _ctx_adjoint_tangent
