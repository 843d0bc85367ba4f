"""ctypes bindings for the CPU oracle (oracle/les_oracle.c) and, when it has
been built in the development container, the compiled reference harness
(oracle/_ref/libles_ref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and
by the CPU-baseline leg of bench.py.  The product library never imports it.

Arrays are numpy float64 / uint8 in the reference layout
idx = i*ny*nz + j*nz + k (les-model src/field.h:40), passed as flat C arrays.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libles_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libles_ref.so")

PC_JACOBI, PC_IC, PC_CHEB, PC_NONE = 0, 1, 2, 3

_dp = C.POINTER(C.c_double)
_u8 = C.POINTER(C.c_uint8)


def build_oracle(force=False):
    """Compiles les_oracle.c into oracle/_build/ (gcc, OpenMP, no FMA)."""
    if os.path.exists(ORACLE_SO) and not force:
        src = os.path.join(HERE, "les_oracle.c")
        if os.path.getmtime(ORACLE_SO) >= max(os.path.getmtime(src),
                                                os.path.getmtime(os.path.join(HERE, "les_oracle.h"))):
            return ORACLE_SO
    os.makedirs(os.path.dirname(ORACLE_SO), exist_ok=True)
    tmp = ORACLE_SO + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
                           "-o", tmp, os.path.join(HERE, "les_oracle.c"), "-lm"])
    os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def build_ref(ref=None):
    """Runs oracle/build_ref.sh on the les-model checkout `ref` (default: the
    REF environment variable; a no-op without a checkout)."""
    env = dict(os.environ)
    if ref:
        env["REF"] = ref
    subprocess.check_call(["bash", os.path.join(HERE, "build_ref.sh")], env=env)
    return REF_SO if os.path.exists(REF_SO) else None


def _p(a):
    if a is None:
        return None
    if a.dtype == np.uint8:
        return a.ctypes.data_as(_u8)
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)



def mt19937_start_vector(n, seed=1337):
    """std::mt19937(seed) + std::uniform_real_distribution<double>(-1, 1) in
    index order: what src/pressure.cpp:926-931 draws on one thread.  The
    legacy numpy RandomState seeds MT19937 with the same init_genrand
    recurrence; generate_canonical<double, 53> combines two 32-bit words as
    (w0 + w1 * 2^32) / 2^64, and the distribution maps u to (b - a) * u + a."""
    words = np.random.RandomState(seed).randint(0, 2 ** 32, size=2 * n, dtype=np.uint32)
    w0 = words[0::2].astype(np.float64)
    w1 = words[1::2].astype(np.float64)
    s = w0 + w1 * 4294967296.0
    u = s / 18446744073709551616.0
    u = np.where(u >= 1.0, np.nextafter(1.0, 0.0), u)
    return 2.0 * u + -1.0

class Mesh(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double)]

    @property
    def n(self):
        return self.nx * self.ny * self.nz

    @property
    def shape(self):
        return (self.nx, self.ny, self.nz)


class _Stencil(C.Structure):
    _fields_ = [(k, _dp) for k in ("c", "n", "s", "e", "w", "t", "b")]


DIAGS = ("c", "n", "s", "e", "w", "t", "b")


def new_stencil(n):
    return {k: np.zeros(n, np.float64) for k in DIAGS}


def _st(d):
    return _Stencil(*[_p(d[k]) for k in DIAGS])


class StepParams(C.Structure):
    _fields_ = [("nu", C.c_double), ("rho", C.c_double), ("cs", C.c_double),
                ("cfl_conv", C.c_double), ("cfl_visc", C.c_double), ("dt_max", C.c_double),
                ("solver", C.c_int), ("pc", C.c_int), ("max_iter", C.c_int),
                ("tol", C.c_double), ("rel_tol", C.c_double), ("omega", C.c_double),
                ("lmin", C.c_double), ("lmax", C.c_double), ("degree", C.c_int),
                ("dt_fixed", C.c_double)]


class _Field(C.Structure):
    _fields_ = [(k, _dp) for k in ("u", "v", "w", "u_new", "v_new", "w_new", "p", "p_rhs", "nu_t")] + \
               [("solid", _u8)]


FIELD_KEYS = ("u", "v", "w", "u_new", "v_new", "w_new", "p", "p_rhs", "nu_t")


class Oracle:
    """The C restatement.  Functions mirror les_oracle.h; arrays are updated in place."""

    def __init__(self, path=None):
        self.lib = C.CDLL(path or build_oracle())
        L = self.lib
        L.lo_dot.restype = C.c_double
        L.lo_norm.restype = C.c_double
        L.lo_compute_adaptive_dt.restype = C.c_double
        L.lo_smagorinsky_coef.restype = C.c_double
        L.lo_lambda_max.restype = C.c_double
        for f in ("lo_solve_jacobi", "lo_solve_gs", "lo_pcg", "lo_step", "lo_get_threads"):
            getattr(L, f).restype = C.c_int
        self.set_threads(1)

    def set_threads(self, n):
        self.lib.lo_set_threads(int(n))

    def threads(self):
        return self.lib.lo_get_threads()

    # --- statistics (src/statistics.cpp)
    def stats_update(self, u, v, w, p, sums):
        arr = (_dp * 10)(*[_p(s) for s in sums])
        self.lib.lo_stats_update(C.c_int64(u.size), _p(u), _p(v), _p(w), _p(p), arr)

    def stats_finalize(self, samples, sums):
        out = [np.empty_like(sums[0]) for _ in range(10)]
        self.lib.lo_stats_finalize(C.c_int64(sums[0].size), C.c_int(samples), (_dp * 10)(*[_p(s) for s in sums]),
                                   (_dp * 10)(*[_p(o) for o in out]))
        return out

    # --- BLAS-1
    def dot(self, a, b):
        return self.lib.lo_dot(C.c_int64(a.size), _p(a), _p(b))

    def norm(self, a):
        return self.lib.lo_norm(C.c_int64(a.size), _p(a))

    # --- physics
    def adaptive_dt(self, m, u, v, w, nu_t, nu, cfl_conv=0.4, cfl_visc=0.2, dt_max=1e-4):
        return self.lib.lo_compute_adaptive_dt(C.byref(m), _p(u), _p(v), _p(w), _p(nu_t),
                                               C.c_double(nu), C.c_double(cfl_conv),
                                               C.c_double(cfl_visc), C.c_double(dt_max))

    def define_obstacle_mask(self, m, solid):
        self.lib.lo_define_obstacle_mask(C.byref(m), _p(solid))

    def velocity_bcs(self, m, u, v, w, solid):
        self.lib.lo_apply_velocity_bcs(C.byref(m), _p(u), _p(v), _p(w), _p(solid))

    def smagorinsky_coef(self, m, cs):
        return self.lib.lo_smagorinsky_coef(C.byref(m), C.c_double(cs))

    def sgs(self, m, cs, u, v, w, nu_t, tau=None):
        self.lib.lo_compute_sgs(C.byref(m), C.c_double(self.smagorinsky_coef(m, cs)), _p(u), _p(v),
                                _p(w), _p(nu_t), _p(tau))

    def nut_bcs(self, m, nu_t, solid):
        self.lib.lo_apply_nut_bcs(C.byref(m), _p(nu_t), _p(solid))

    def momentum(self, m, dt, nu, u, v, w, nu_t, un, vn, wn):
        self.lib.lo_solve_momentum(C.byref(m), C.c_double(dt), C.c_double(nu), _p(u), _p(v), _p(w),
                                   _p(nu_t), _p(un), _p(vn), _p(wn))

    def correct_velocity(self, m, dt, rho, p, u, v, w):
        self.lib.lo_correct_velocity(C.byref(m), C.c_double(dt), C.c_double(rho), _p(p), _p(u),
                                     _p(v), _p(w))

    # --- pressure
    def pressure_bcs(self, m, p, solid):
        self.lib.lo_apply_pressure_bcs(C.byref(m), _p(p), _p(solid))

    def solve_jacobi(self, m, dt, rho, u, v, w, p, solid, max_iter=100, tol=1e-6):
        return self.lib.lo_solve_jacobi(C.byref(m), C.c_double(dt), C.c_double(rho), _p(u), _p(v),
                                        _p(w), _p(p), _p(solid), int(max_iter), C.c_double(tol))

    def solve_gs(self, m, dt, rho, u, v, w, p, solid, max_iter=200, omega=1.7, tol=1e-6):
        return self.lib.lo_solve_gs(C.byref(m), C.c_double(dt), C.c_double(rho), _p(u), _p(v), _p(w),
                                    _p(p), _p(solid), int(max_iter), C.c_double(omega),
                                    C.c_double(tol))

    def divergence(self, m, dt, rho, un, vn, wn, solid, rhs):
        self.lib.lo_calculate_divergence(C.byref(m), C.c_double(dt), C.c_double(rho), _p(un), _p(vn),
                                         _p(wn), _p(solid), _p(rhs))

    def build_b(self, m, div, solid, b):
        self.lib.lo_build_b(C.byref(m), _p(div), _p(solid), _p(b))

    def build_stencil(self, m, solid):
        A = new_stencil(m.n)
        self.lib.lo_build_stencil(C.byref(m), _p(solid), C.byref(_st(A)))
        return A

    def spmv(self, m, A, p, q):
        self.lib.lo_spmv(C.byref(m), C.byref(_st(A)), _p(p), _p(q))

    def jacobi_precond(self, A, r, z):
        self.lib.lo_jacobi_precond(C.c_int64(r.size), C.byref(_st(A)), _p(r), _p(z))

    def ic_build(self, m, A):
        L = new_stencil(m.n)
        self.lib.lo_ic_build(C.byref(m), C.byref(_st(A)), C.byref(_st(L)))
        return L

    def ic_apply(self, m, L, r, z):
        self.lib.lo_ic_apply(C.byref(m), C.byref(_st(L)), _p(r), _p(z))

    def cheb_apply(self, m, A, lmin, lmax, degree, r, z):
        wp = np.zeros(m.n)
        wr = np.zeros(m.n)
        self.lib.lo_cheb_apply(C.byref(m), C.byref(_st(A)), C.c_double(lmin), C.c_double(lmax),
                               int(degree), _p(r), _p(z), _p(wp), _p(wr))

    def lambda_max(self, m, A, v0, n_iter=20):
        wv = np.zeros(m.n)
        ww = np.zeros(m.n)
        return self.lib.lo_lambda_max(C.byref(m), C.byref(_st(A)), _p(v0), int(n_iter), _p(wv), _p(ww))

    def pcg(self, m, A, b, x, pc, L=None, lmin=0.0, lmax=0.0, degree=4, max_iter=1000, tol=1e-6):
        work = np.zeros(4 * m.n)
        fn = C.c_double(0)
        it = self.lib.lo_pcg(C.byref(m), C.byref(_st(A)), _p(b), _p(x), int(pc),
                             C.byref(_st(L)) if L is not None else None, C.c_double(lmin),
                             C.c_double(lmax), int(degree), int(max_iter), C.c_double(tol),
                             _p(work), C.byref(fn))
        return it, fn.value

    def step(self, m, f, A, L, prm):
        """f: dict of numpy arrays FIELD_KEYS + 'solid'.  Swaps u<->u_new entries
        in the dict like the reference's vector swap.  Returns (iters, dt)."""
        cf = _Field(*[_p(f[k]) for k in FIELD_KEYS], _p(f["solid"]))
        b = np.zeros(m.n)
        work = np.zeros(4 * m.n)
        dt = C.c_double(0)
        it = self.lib.lo_step(C.byref(m), C.byref(cf), C.byref(_st(A)),
                              C.byref(_st(L)) if L is not None else None, C.byref(prm), _p(b),
                              _p(work), C.byref(dt))
        # the C side swapped pointers; mirror that on the dict
        addr = {f[k].ctypes.data: k for k in FIELD_KEYS}
        newf = {}
        for k in FIELD_KEYS:
            newf[k] = f[addr[C.cast(getattr(cf, k), C.c_void_p).value]]
        f.update(newf)
        return it, dt.value


class Ref:
    """The compiled reference (oracle/_ref/libles_ref.so), development container only."""

    def __init__(self, path=REF_SO):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = C.CDLL(path)
        L = self.lib
        for f in ("ref_adaptive_dt", "ref_lambda_max"):
            getattr(L, f).restype = C.c_double
        for f in ("ref_pcg_shipped", "ref_pcg_cheb", "ref_pcg_restated", "ref_step"):
            getattr(L, f).restype = C.c_int
        self.set_threads(1)

    def set_threads(self, n):
        self.lib.ref_set_threads(int(n))

    @staticmethod
    def _m(m):
        return (C.c_int(m.nx), C.c_int(m.ny), C.c_int(m.nz), C.c_double(m.dx), C.c_double(m.dy),
                C.c_double(m.dz))

    @staticmethod
    def _d(A):
        return (_dp * 7)(*[_p(A[k]) for k in DIAGS])

    def __getattr__(self, name):
        fn = getattr(self.lib, "ref_" + name)

        def call(m, *args):
            conv = []
            for a in args:
                if isinstance(a, np.ndarray):
                    conv.append(_p(a))
                elif isinstance(a, dict):
                    conv.append(self._d(a))
                elif a is None:
                    conv.append(None)
                elif isinstance(a, float):
                    conv.append(C.c_double(a))
                elif isinstance(a, int):
                    conv.append(C.c_int(a))
                else:
                    conv.append(a)
            return fn(*self._m(m), *conv)

        return call
