"""ctypes binding of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and the cpu_baseline / --impl reference
legs of bench.py import this module.  It loads oracle/_build/libtea_oracle.so,
building it with gcc first if needed.
"""
import ctypes as C
import os

# many short parallel regions: sleeping idle threads keep a shared or
# oversubscribed host usable
os.environ.setdefault("OMP_WAIT_POLICY", "PASSIVE")

import numpy as np

from . import build as _build

FIELD = dict(density=1, energy0=2, energy1=3, u=4, p=5, sd=6, r=7, u0=8, w=9,
             z=10, Mi=11, Kx=12, Ky=13, cp=14, bfp=15, volume=16)


class OracleResult(C.Structure):
    _fields_ = [
        ("n_summaries", C.c_int),
        ("n_steps", C.c_int),
        ("summary", (C.c_double * 6) * 64),
        ("iterations", C.c_int * 1024),
        ("inner_iterations", C.c_int * 1024),
        ("conduction_error", C.c_double * 1024),
        ("exact_error", C.c_double * 1024),
        ("final_temp", C.c_double),
        ("solve_seconds", C.c_double),
        ("step_seconds", C.c_double * 1024),
        ("total_outer_iterations", C.c_longlong),
        ("total_inner_iterations", C.c_longlong),
        ("qa_passed", C.c_int),
        ("qa_diff", C.c_double),
        ("outer_corrections", C.c_int * 1024),
        ("relative_residual", C.c_double * 1024),
        ("switch_iteration", C.c_int * 1024),
    ]

    def summaries(self):
        n = min(self.n_summaries, 64)
        start = self.n_summaries - n
        rows = [list(self.summary[(start + i) % 64]) for i in range(n)]
        return np.array(rows)


class MixedInfo(C.Structure):
    _fields_ = [
        ("outer_iterations", C.c_int), ("inner_iterations", C.c_longlong),
        ("initial_residual", C.c_double), ("final_residual", C.c_double),
        ("relative_residual", C.c_double), ("ppcg_inner_steps", C.c_longlong),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        d, i, pd, pi = C.c_double, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_int)
        sig = {
            "oracle_initialise": (i, [i, i, i, i, i]),
            "oracle_finalise": (None, []),
            "oracle_initialise_chunk": (None, [d, d, d, d]),
            "oracle_generate_chunk": (None, [i, pd, pd, pd, pd, pd, pd, pd, pi]),
            "oracle_set_field": (None, []),
            "oracle_common_init": (None, [i, d, pd, pd, pi, i]),
            "oracle_calc_residual": (None, []),
            "oracle_calc_2norm": (None, [i, pd]),
            "oracle_cg_init": (None, [pd]),
            "oracle_cg_calc_w": (None, [pd]),
            "oracle_cg_calc_ur": (None, [d, pd]),
            "oracle_cg_calc_p": (None, [d]),
            "oracle_cheby_init": (None, [pd, pd, i, d]),
            "oracle_cheby_iterate": (None, [i]),
            "oracle_ppcg_init": (None, [pd, pd, d, i]),
            "oracle_ppcg_init_sd": (None, []),
            "oracle_ppcg_inner": (None, [i]),
            "oracle_jacobi_solve": (None, [pd]),
            "oracle_finalise_kernel": (None, []),
            "oracle_field_summary": (None, [pd, pd, pd, pd]),
            "oracle_update_halo": (None, [pi, i]),
            "oracle_read_field": (i, [i, pd]),
            "oracle_write_field": (i, [i, pd]),
            "oracle_read_field_padded": (i, [i, pd, C.c_long]),
            "oracle_write_field_padded": (i, [i, pd, C.c_long]),
            "oracle_reduce": (d, [pd, i, i]),
            "oracle_reduce_pairs": (d, [pd, pd, i, i, i]),
            "oracle_set_arithmetic": (None, [i]),
            "oracle_get_arithmetic": (i, []),
            "oracle_reduction_rows": (i, [i, i]),
            "oracle_run_deck": (i, [C.c_char_p, C.c_char_p, i, i,
                                    C.POINTER(OracleResult), C.c_char_p, i]),
            "oracle_num_threads": (i, []),
            "oracle_mixed_solve": (i, [d, d, i, i, C.POINTER(MixedInfo)]),
            "oracle_mixed_solve_ppcg": (i, [d, d, i, i, i, i, C.POINTER(MixedInfo)]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _pd(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def run_deck(deck_text, log_path=None, max_solver_iters=0, max_after_switch=0):
    """Run a tea.in deck on the oracle; returns an OracleResult.
    max_solver_iters > 0 caps every step's solver iterations;
    max_after_switch > 0 ends each Chebyshev/PPCG step that many iterations
    after its switch from CG (the switch's own iteration counted)."""
    res = OracleResult()
    err = C.create_string_buffer(512)
    rc = lib().oracle_run_deck(deck_text.encode(),
                               log_path.encode() if log_path else None,
                               int(max_solver_iters), int(max_after_switch),
                               C.byref(res), err, 512)
    if rc != 0:
        raise RuntimeError("oracle run failed: " + err.value.decode())
    return res


def reduce(contrib):
    a = np.ascontiguousarray(contrib, dtype=np.float64)
    return lib().oracle_reduce(_pd(a), a.shape[1], a.shape[0])


def reduce_pairs(a, b, fused):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    return lib().oracle_reduce_pairs(_pd(a), _pd(b), a.shape[1], a.shape[0], int(fused))


class Chunk:
    """Per-call access to the oracle chunk, mirroring the C-ABI entry points."""

    def __init__(self, x_max, y_max, halo, solver, prec):
        rc = lib().oracle_initialise(x_max, y_max, halo, solver, prec)
        if rc != 0:
            raise RuntimeError("oracle_initialise failed %d" % rc)
        self.x_max, self.y_max, self.halo = x_max, y_max, halo

    def set_arithmetic(self, form):
        """0/False exact, 1/True fused, 2 chain (or the names)."""
        if isinstance(form, str):
            form = dict(exact=0, fused=1, chain=2)[form]
        lib().oracle_set_arithmetic(int(form))

    # -- the same entry points as tealeaf_opencl_gb300.lib.Chunk -------------
    def initialise_chunk(self, xmin, ymin, dx, dy):
        lib().oracle_initialise_chunk(xmin, ymin, dx, dy)

    def generate_chunk(self, density, energy, xmin, xmax, ymin, ymax, radius, geometry):
        arrs = [np.ascontiguousarray(a, dtype=np.float64)
                for a in (density, energy, xmin, xmax, ymin, ymax, radius)]
        geom = np.ascontiguousarray(geometry, dtype=np.int32)
        lib().oracle_generate_chunk(len(geom), *[_pd(a) for a in arrs],
                                    geom.ctypes.data_as(C.POINTER(C.c_int)))

    def set_field(self):
        lib().oracle_set_field()

    def common_init(self, coefficient, dt, zero_boundary=(1, 1, 1, 1), reflective=0):
        rx, ry = C.c_double(), C.c_double()
        zb = np.ascontiguousarray(zero_boundary, dtype=np.int32)
        lib().oracle_common_init(int(coefficient), float(dt), C.byref(rx), C.byref(ry),
                                 zb.ctypes.data_as(C.POINTER(C.c_int)), int(reflective))
        return rx.value, ry.value

    def calc_residual(self):
        lib().oracle_calc_residual()

    def _scalar(self, fn, *args):
        out = C.c_double()
        fn(*args, C.byref(out))
        return out.value

    def calc_2norm(self, which):
        return self._scalar(lib().oracle_calc_2norm, int(which))

    def cg_init(self):
        return self._scalar(lib().oracle_cg_init)

    def cg_calc_w(self):
        return self._scalar(lib().oracle_cg_calc_w)

    def cg_calc_ur(self, alpha):
        return self._scalar(lib().oracle_cg_calc_ur, float(alpha))

    def cg_calc_p(self, beta):
        lib().oracle_cg_calc_p(float(beta))

    def cheby_init(self, alphas, betas, theta, rx=0.0, ry=0.0):
        a = np.ascontiguousarray(alphas, dtype=np.float64)
        b = np.ascontiguousarray(betas, dtype=np.float64)
        lib().oracle_cheby_init(_pd(a), _pd(b), len(a), float(theta))

    def cheby_iterate(self, step):
        lib().oracle_cheby_iterate(int(step))

    def ppcg_init(self, alphas, betas, theta):
        a = np.ascontiguousarray(alphas, dtype=np.float64)
        b = np.ascontiguousarray(betas, dtype=np.float64)
        lib().oracle_ppcg_init(_pd(a), _pd(b), float(theta), len(a))

    def ppcg_init_sd(self):
        lib().oracle_ppcg_init_sd()

    def ppcg_inner(self, step, bounds_extra=0):
        lib().oracle_ppcg_inner(int(step))

    def jacobi_solve(self):
        return self._scalar(lib().oracle_jacobi_solve)

    def finalise(self):
        lib().oracle_finalise_kernel()

    def field_summary(self):
        out = [C.c_double() for _ in range(4)]
        lib().oracle_field_summary(*[C.byref(o) for o in out])
        return tuple(o.value for o in out)

    def mixed_solve(self, tol, inner_tol=1e-4, max_outer=50, max_inner=10000):
        info = MixedInfo()
        if lib().oracle_mixed_solve(tol, inner_tol, max_outer, max_inner, C.byref(info)) != 0:
            raise RuntimeError("oracle mixed solve failed")
        return info

    def mixed_solve_ppcg(self, tol, inner_tol=1e-4, max_outer=50, max_inner=10000,
                         presteps=25, inner_steps=10):
        info = MixedInfo()
        if lib().oracle_mixed_solve_ppcg(tol, inner_tol, max_outer, max_inner, presteps,
                                         inner_steps, C.byref(info)) != 0:
            raise RuntimeError("oracle mixed PPCG solve failed")
        return info

    def update_halo(self, fields, depth):
        f = np.ascontiguousarray(fields, dtype=np.int32)
        lib().oracle_update_halo(f.ctypes.data_as(C.POINTER(C.c_int)), int(depth))

    # -- field access ----------------------------------------------------------
    def read(self, name):
        out = np.zeros((self.y_max, self.x_max))
        if lib().oracle_read_field(FIELD[name], _pd(out)) != 0:
            raise KeyError(name)
        return out

    def write(self, name, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        assert a.shape == (self.y_max, self.x_max)
        if lib().oracle_write_field(FIELD[name], _pd(a)) != 0:
            raise KeyError(name)

    def read_padded(self, name):
        xs, ys = self.x_max + 2 * self.halo, self.y_max + 2 * self.halo
        out = np.zeros((ys, xs))
        if lib().oracle_read_field_padded(FIELD[name], _pd(out), out.size) != 0:
            raise KeyError(name)
        return out

    def write_padded(self, name, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        if lib().oracle_write_field_padded(FIELD[name], _pd(a), a.size) != 0:
            raise KeyError(name)
