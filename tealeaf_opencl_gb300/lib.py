"""ctypes binding of libtealeaf_gb300.so (the C ABI in include/tealeaf_gb300.h).

The library is the product: every call here goes to hand-written CUDA
kernels for sm_103a.  There is no CPU fallback; if the shared library is
missing and cannot be built, load() raises.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

FIELD = dict(density=1, energy0=2, energy1=3, u=4, p=5, sd=6, r=7, u0=8, w=9,
             z=10, Mi=11, Kx=12, Ky=13, cp=14, bfp=15, volume=16)
PREC = dict(none=1, jac_diag=2, jac_block=3)
SOLVER = dict(jacobi=1, cg=2, chebyshev=3, ppcg=4)
EXTERNAL_FACE = -1
DRIVER_PER_CALL = 0
DRIVER_RESIDENT = 1
CHECK_BREAKDOWN = 1  # TEA_CHECK_BREAKDOWN
CHECK_MAX_ITERS = 2  # TEA_CHECK_MAX_ITERS

# the C-ABI entry points declared in include/tealeaf_gb300.h
REFERENCE_SYMBOLS = [
    "initialise_ocl_", "initialise_chunk_kernel_ocl_", "generate_chunk_kernel_ocl_",
    "set_field_kernel_ocl_", "field_summary_kernel_ocl_", "update_halo_kernel_ocl_",
    "tea_leaf_common_init_kernel_ocl_", "tea_leaf_calc_residual_ocl_",
    "tea_leaf_calc_2norm_kernel_ocl_", "tea_leaf_cg_init_kernel_ocl_",
    "tea_leaf_cg_calc_w_kernel_ocl_", "tea_leaf_cg_calc_ur_kernel_ocl_",
    "tea_leaf_cg_calc_p_kernel_ocl_", "tea_leaf_cheby_init_kernel_ocl_",
    "tea_leaf_cheby_iterate_kernel_ocl_", "tea_leaf_ppcg_init_ocl_",
    "tea_leaf_ppcg_init_sd_kernel_ocl_", "tea_leaf_ppcg_inner_kernel_ocl_",
    "tea_leaf_jacobi_solve_kernel_ocl_", "tea_leaf_common_finalise_kernel_ocl_",
    "print_opencl_profiling_info_", "ocl_pack_buffers_", "ocl_unpack_buffers_",
]
EXTRA_SYMBOLS = [
    "tea_gb300_configure", "tea_gb300_set_arithmetic", "tea_gb300_get_arithmetic",
    "tea_gb300_set_resident_mode", "tea_gb300_set_barrier_limits", "tea_gb300_set_inner_pairs",
    "tea_gb300_set_abort_on_error", "tea_gb300_last_error",
    "tea_gb300_finalise", "tea_gb300_read_field", "tea_gb300_write_field",
    "tea_gb300_read_field_padded", "tea_gb300_write_field_padded",
    "tea_gb300_reduction_rows", "tea_gb300_kernel_launches", "tea_gb300_stream",
    "tea_gb300_chunk_info", "tea_gb300_event_record", "tea_gb300_event_elapsed_ms",
    "tea_gb300_synchronize", "tea_gb300_host_alloc", "tea_gb300_host_free",
    "tea_gb300_kernel_timer_select", "tea_gb300_kernel_timer_read",
    "tea_gb300_kernel_timer_read_name", "tea_gb300_fp64_rate", "tea_gb300_emu_check",
    "tea_gb300_dot_noalloc", "tea_gb300_mixed_solve", "tea_gb300_mixed_solve_ppcg",
    "tea_gb300_driver_open", "tea_gb300_driver_step", "tea_gb300_driver_close",
    "tea_gb300_driver_set_limits",
    "tea_gb300_batch_create", "tea_gb300_batch_set_fields", "tea_gb300_batch_run",
    "tea_gb300_batch_summary", "tea_gb300_batch_iterations",
    "tea_gb300_batch_read_field", "tea_gb300_batch_set_launch",
    "tea_gb300_batch_get_launch", "tea_gb300_batch_autotune", "tea_gb300_batch_free",
    "tea_gb300_adjoint_create", "tea_gb300_adjoint_forward", "tea_gb300_adjoint_backward",
    "tea_gb300_adjoint_free",
]


class StepInfo(C.Structure):
    _fields_ = [
        ("step", C.c_int), ("time", C.c_double), ("dt", C.c_double),
        ("iterations", C.c_int), ("inner_iterations", C.c_int),
        ("conduction_error", C.c_double), ("exact_error", C.c_double),
        ("summary_done", C.c_int), ("vol", C.c_double), ("mass", C.c_double),
        ("ie", C.c_double), ("temp", C.c_double), ("complete", C.c_int),
        ("qa_passed", C.c_int), ("qa_diff", C.c_double),
        ("outer_corrections", C.c_int), ("relative_residual", C.c_double),
        ("switch_iteration", C.c_int),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class MixedInfo(C.Structure):
    _fields_ = [
        ("outer_iterations", C.c_int), ("inner_iterations", C.c_longlong),
        ("initial_residual", C.c_double), ("final_residual", C.c_double),
        ("relative_residual", C.c_double), ("ppcg_inner_steps", C.c_longlong),
    ]


ARITHMETIC = dict(exact=0, fused=1, chain=2)


def arithmetic_form(form):
    """Arithmetic form number from a name, a bool (fused or not) or a number."""
    if isinstance(form, str):
        return ARITHMETIC[form]
    return int(form)


class BatchStats(C.Structure):
    _fields_ = [
        ("steps", C.c_int), ("max_iterations", C.c_int), ("iterations", C.c_longlong),
        ("cell_iterations", C.c_double), ("graph_launches", C.c_int),
        ("kernel_launches", C.c_longlong), ("solve_ms", C.c_double),
        ("total_ms", C.c_double),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class BatchLaunch(C.Structure):
    _fields_ = [("blocks_per_sm", C.c_int), ("graph_iterations", C.c_int),
                ("supertiles_per_unit", C.c_int), ("persistent", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class AdjointConfig(C.Structure):
    _fields_ = [("steps", C.c_int), ("dt", C.c_double), ("eps", C.c_double),
                ("max_iters", C.c_int), ("checkpoint_every", C.c_int)]


class AdjointStats(C.Structure):
    _fields_ = [
        ("forward_iterations", C.c_longlong), ("recompute_iterations", C.c_longlong),
        ("adjoint_iterations", C.c_longlong), ("checkpoints", C.c_int),
        ("forward_ms", C.c_double), ("backward_ms", C.c_double),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class TeaError(RuntimeError):
    pass


_lib = None
PI = C.POINTER(C.c_int)
PD = C.POINTER(C.c_double)


def library_path():
    return _build.LIB


def load(build=True):
    """Load the CUDA library (building it with nvcc first if needed)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.build() if build else _build.LIB
    if not os.path.exists(path):
        raise TeaError("libtealeaf_gb300.so not found at %s" % path)
    L = C.CDLL(path)
    d, i, v = C.c_double, C.c_int, None
    sig = {
        "initialise_ocl_": (v, [PI, PI, PI, PI]),
        "initialise_chunk_kernel_ocl_": (v, [PD, PD, PD, PD]),
        "generate_chunk_kernel_ocl_": (v, [PI, PD, PD, PD, PD, PD, PD, PD, PI, PI, PI, PI]),
        "set_field_kernel_ocl_": (v, []),
        "field_summary_kernel_ocl_": (v, [PD, PD, PD, PD]),
        "update_halo_kernel_ocl_": (v, [PI, PI, PI]),
        "tea_leaf_common_init_kernel_ocl_": (v, [PI, PD, PD, PD, PI, PI]),
        "tea_leaf_calc_residual_ocl_": (v, []),
        "tea_leaf_calc_2norm_kernel_ocl_": (v, [PI, PD]),
        "tea_leaf_cg_init_kernel_ocl_": (v, [PD]),
        "tea_leaf_cg_calc_w_kernel_ocl_": (v, [PD]),
        "tea_leaf_cg_calc_ur_kernel_ocl_": (v, [PD, PD]),
        "tea_leaf_cg_calc_p_kernel_ocl_": (v, [PD]),
        "tea_leaf_cheby_init_kernel_ocl_": (v, [PD, PD, PI, PD, PD, PD]),
        "tea_leaf_cheby_iterate_kernel_ocl_": (v, [PI]),
        "tea_leaf_ppcg_init_ocl_": (v, [PD, PD, PD, PI]),
        "tea_leaf_ppcg_init_sd_kernel_ocl_": (v, []),
        "tea_leaf_ppcg_inner_kernel_ocl_": (v, [PI, PI, PI]),
        "tea_leaf_jacobi_solve_kernel_ocl_": (v, [PD]),
        "tea_leaf_common_finalise_kernel_ocl_": (v, []),
        "print_opencl_profiling_info_": (v, []),
        "ocl_pack_buffers_": (v, [PI, PI, PI, PI, PD]),
        "ocl_unpack_buffers_": (v, [PI, PI, PI, PI, PD]),
        "tea_gb300_configure": (i, [i, i, i, i]),
        "tea_gb300_set_abort_on_error": (v, [i]),
        "tea_gb300_set_arithmetic": (i, [i]),
        "tea_gb300_get_arithmetic": (i, []),
        "tea_gb300_set_resident_mode": (i, [i]),
        "tea_gb300_set_barrier_limits": (i, [C.c_longlong, i]),
        "tea_gb300_set_inner_pairs": (i, [i]),
        "tea_gb300_last_error": (i, [C.c_char_p, i]),
        "tea_gb300_finalise": (v, []),
        "tea_gb300_read_field": (i, [i, PD]),
        "tea_gb300_write_field": (i, [i, PD]),
        "tea_gb300_read_field_padded": (i, [i, PD]),
        "tea_gb300_write_field_padded": (i, [i, PD]),
        "tea_gb300_reduction_rows": (i, [i, i]),
        "tea_gb300_kernel_launches": (C.c_longlong, []),
        "tea_gb300_stream": (C.c_void_p, []),
        "tea_gb300_chunk_info": (i, [PI, PI, PI, PI]),
        "tea_gb300_event_record": (i, [i]),
        "tea_gb300_event_elapsed_ms": (C.c_float, [i, i]),
        "tea_gb300_synchronize": (i, []),
        "tea_gb300_host_alloc": (C.c_void_p, [C.c_size_t]),
        "tea_gb300_host_free": (v, [C.c_void_p]),
        "tea_gb300_kernel_timer_select": (i, [C.c_char_p]),
        "tea_gb300_kernel_timer_read": (i, [PD, C.POINTER(C.c_longlong)]),
        "tea_gb300_kernel_timer_read_name": (i, [C.c_char_p, PD, C.POINTER(C.c_longlong)]),
        "tea_gb300_fp64_rate": (d, []),
        "tea_gb300_emu_check": (i, [i, C.c_void_p, C.c_void_p, C.c_longlong, d,
                                    C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
        "tea_gb300_dot_noalloc": (i, [C.c_void_p, C.c_void_p, i, i, i, C.c_longlong,
                                      C.c_void_p, C.c_void_p]),
        "tea_gb300_mixed_solve": (i, [d, d, i, i, C.POINTER(MixedInfo)]),
        "tea_gb300_mixed_solve_ppcg": (i, [d, d, i, i, i, i, C.POINTER(MixedInfo)]),
        "tea_gb300_driver_open": (i, [C.c_char_p, C.c_char_p, i, i]),
        "tea_gb300_driver_step": (i, [C.POINTER(StepInfo)]),
        "tea_gb300_driver_close": (v, []),
        "tea_gb300_driver_set_limits": (i, [i, i]),
        "tea_gb300_batch_create": (i, [i, PI, PI, d, d, d, d, i, i]),
        "tea_gb300_batch_set_fields": (i, [i, PD, PD]),
        "tea_gb300_batch_run": (i, [i, d, d, i, C.POINTER(BatchStats)]),
        "tea_gb300_batch_summary": (i, [i, PD]),
        "tea_gb300_batch_iterations": (i, [i, PI, i]),
        "tea_gb300_batch_read_field": (i, [i, i, PD]),
        "tea_gb300_batch_set_launch": (i, [C.POINTER(BatchLaunch)]),
        "tea_gb300_batch_get_launch": (i, [C.POINTER(BatchLaunch)]),
        "tea_gb300_batch_autotune": (i, [C.POINTER(BatchLaunch)]),
        "tea_gb300_batch_free": (v, []),
        "tea_gb300_adjoint_create": (i, [i, i, d, d, d, d, i, i]),
        "tea_gb300_adjoint_forward": (i, [C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.POINTER(AdjointConfig), PD, C.c_void_p,
                                          C.POINTER(AdjointStats)]),
        "tea_gb300_adjoint_backward": (i, [C.c_void_p, C.POINTER(AdjointStats)]),
        "tea_gb300_adjoint_free": (v, []),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    L.tea_gb300_set_abort_on_error(0)
    _lib = L
    return L


def check():
    """Raise TeaError if the library recorded an error since the last check."""
    buf = C.create_string_buffer(1024)
    code = load().tea_gb300_last_error(buf, 1024)
    if code:
        raise TeaError("libtealeaf_gb300 error %d: %s" % (code, buf.value.decode()))


def _ip(v):
    return C.byref(C.c_int(int(v)))


def _dp(v):
    return C.byref(C.c_double(float(v)))


def _pd(a):
    return a.ctypes.data_as(PD)


def _pi(a):
    return a.ctypes.data_as(PI)


class Chunk:
    """The process-global chunk, driven through the reference's entry points."""

    def __init__(self, x_max, y_max, halo=1, solver="cg", prec="none", profiler=False):
        L = load()
        s = SOLVER[solver] if isinstance(solver, str) else int(solver)
        p = PREC[prec] if isinstance(prec, str) else int(prec)
        if L.tea_gb300_configure(int(halo), s, p, 1 if profiler else 0) != 0:
            raise TeaError("invalid configuration")
        L.initialise_ocl_(_ip(1), _ip(x_max), _ip(1), _ip(y_max))
        check()
        self.x_max, self.y_max, self.halo = x_max, y_max, halo
        self.neighbours = np.full(4, EXTERNAL_FACE, dtype=np.int32)

    def set_arithmetic(self, form):
        """0/False exact, 1/True fused, 2 chain (or the names)."""
        load().tea_gb300_set_arithmetic(arithmetic_form(form))

    # -- setup -------------------------------------------------------------
    def initialise_chunk(self, xmin, ymin, dx, dy):
        load().initialise_chunk_kernel_ocl_(_dp(xmin), _dp(ymin), _dp(dx), _dp(dy))
        check()

    def generate_chunk(self, density, energy, xmin, xmax, ymin, ymax, radius, geometry):
        arrs = [np.ascontiguousarray(a, dtype=np.float64)
                for a in (density, energy, xmin, xmax, ymin, ymax, radius)]
        geom = np.ascontiguousarray(geometry, dtype=np.int32)
        load().generate_chunk_kernel_ocl_(_ip(len(geom)), *[_pd(a) for a in arrs],
                                          _pi(geom), _ip(1), _ip(2), _ip(3))
        check()

    def set_field(self):
        load().set_field_kernel_ocl_()
        check()

    # -- solver entry points -----------------------------------------------
    def common_init(self, coefficient, dt, zero_boundary=(1, 1, 1, 1), reflective=0):
        rx, ry = C.c_double(), C.c_double()
        zb = np.ascontiguousarray(zero_boundary, dtype=np.int32)
        load().tea_leaf_common_init_kernel_ocl_(_ip(coefficient), _dp(dt), C.byref(rx),
                                                C.byref(ry), _pi(zb), _ip(reflective))
        check()
        return rx.value, ry.value

    def calc_residual(self):
        load().tea_leaf_calc_residual_ocl_()
        check()

    def _scalar(self, fn, *args):
        out = C.c_double()
        fn(*args, C.byref(out))
        check()
        return out.value

    def calc_2norm(self, which):
        return self._scalar(load().tea_leaf_calc_2norm_kernel_ocl_, _ip(which))

    def cg_init(self):
        return self._scalar(load().tea_leaf_cg_init_kernel_ocl_)

    def cg_calc_w(self):
        return self._scalar(load().tea_leaf_cg_calc_w_kernel_ocl_)

    def cg_calc_ur(self, alpha):
        return self._scalar(load().tea_leaf_cg_calc_ur_kernel_ocl_, _dp(alpha))

    def cg_calc_p(self, beta):
        load().tea_leaf_cg_calc_p_kernel_ocl_(_dp(beta))
        check()

    def cheby_init(self, alphas, betas, theta, rx=0.0, ry=0.0):
        a = np.ascontiguousarray(alphas, dtype=np.float64)
        b = np.ascontiguousarray(betas, dtype=np.float64)
        load().tea_leaf_cheby_init_kernel_ocl_(_pd(a), _pd(b), _ip(len(a)), _dp(rx),
                                               _dp(ry), _dp(theta))
        check()

    def cheby_iterate(self, step):
        load().tea_leaf_cheby_iterate_kernel_ocl_(_ip(step))
        check()

    def ppcg_init(self, alphas, betas, theta):
        a = np.ascontiguousarray(alphas, dtype=np.float64)
        b = np.ascontiguousarray(betas, dtype=np.float64)
        load().tea_leaf_ppcg_init_ocl_(_pd(a), _pd(b), _dp(theta), _ip(len(a)))
        check()

    def ppcg_init_sd(self):
        load().tea_leaf_ppcg_init_sd_kernel_ocl_()
        check()

    def ppcg_inner(self, step, bounds_extra=0):
        load().tea_leaf_ppcg_inner_kernel_ocl_(_ip(step), _ip(bounds_extra),
                                               _pi(self.neighbours))
        check()

    def jacobi_solve(self):
        return self._scalar(load().tea_leaf_jacobi_solve_kernel_ocl_)

    def finalise(self):
        load().tea_leaf_common_finalise_kernel_ocl_()
        check()

    def field_summary(self):
        out = [C.c_double() for _ in range(4)]
        load().field_summary_kernel_ocl_(*[C.byref(o) for o in out])
        check()
        return tuple(o.value for o in out)

    def mixed_solve(self, tol, inner_tol=1e-4, max_outer=50, max_inner=10000):
        info = MixedInfo()
        if load().tea_gb300_mixed_solve(tol, inner_tol, max_outer, max_inner,
                                        C.byref(info)) != 0:
            check()
            raise TeaError("mixed solve failed")
        return info

    def mixed_solve_ppcg(self, tol, inner_tol=1e-4, max_outer=50, max_inner=10000,
                         presteps=25, inner_steps=10):
        info = MixedInfo()
        if load().tea_gb300_mixed_solve_ppcg(tol, inner_tol, max_outer, max_inner, presteps,
                                             inner_steps, C.byref(info)) != 0:
            check()
            raise TeaError("mixed PPCG solve failed")
        return info

    def update_halo(self, fields, depth):
        f = np.ascontiguousarray(fields, dtype=np.int32)
        load().update_halo_kernel_ocl_(_pi(self.neighbours), _pi(f), _ip(depth))
        check()

    # -- field access -------------------------------------------------------
    def read(self, name):
        out = np.zeros((self.y_max, self.x_max))
        if load().tea_gb300_read_field(FIELD[name], _pd(out)) != 0:
            check()
        return out

    def write(self, name, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        assert a.shape == (self.y_max, self.x_max)
        if load().tea_gb300_write_field(FIELD[name], _pd(a)) != 0:
            check()

    def read_padded(self, name):
        out = np.zeros((self.y_max + 2 * self.halo, self.x_max + 2 * self.halo))
        if load().tea_gb300_read_field_padded(FIELD[name], _pd(out)) != 0:
            check()
        return out

    def write_padded(self, name, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        assert a.shape == (self.y_max + 2 * self.halo, self.x_max + 2 * self.halo)
        if load().tea_gb300_write_field_padded(FIELD[name], _pd(a)) != 0:
            check()


def chunk_shape():
    """(x_max, y_max, halo, stride) of the current chunk."""
    v = [C.c_int() for _ in range(4)]
    if load().tea_gb300_chunk_info(*[C.byref(x) for x in v]) != 0:
        raise TeaError("no chunk")
    return tuple(x.value for x in v)


def read_field(name):
    """Interior of a field of the current chunk (y_max x x_max)."""
    x, y, _, _ = chunk_shape()
    out = np.zeros((y, x))
    if load().tea_gb300_read_field(FIELD[name], _pd(out)) != 0:
        check()
    return out


def write_field(name, arr):
    x, y, _, _ = chunk_shape()
    a = np.ascontiguousarray(arr, dtype=np.float64)
    assert a.shape == (y, x)
    if load().tea_gb300_write_field(FIELD[name], _pd(a)) != 0:
        check()


class Driver:
    """The whole-run driver: tea.in text in, one timestep per step()."""

    def __init__(self, deck_text, mode=DRIVER_PER_CALL, max_iters_cap=0, log_path=None,
                 cap_after_switch=0, checks=0):
        L = load()
        rc = L.tea_gb300_driver_open(deck_text.encode(),
                                     log_path.encode() if log_path else None,
                                     int(mode), int(max_iters_cap))
        if rc != 0:
            check()
            raise TeaError("driver_open failed")
        if (cap_after_switch or checks) and \
                L.tea_gb300_driver_set_limits(int(cap_after_switch), int(checks)) != 0:
            check()
            raise TeaError("driver_set_limits failed")

    def step(self):
        info = StepInfo()
        rc = load().tea_gb300_driver_step(C.byref(info))
        if rc < 0:
            check()
            raise TeaError("driver_step failed")
        return None if rc == 1 else info

    def close(self):
        load().tea_gb300_driver_close()


def run_deck(deck_text, mode=DRIVER_PER_CALL, max_iters_cap=0, log_path=None,
             cap_after_switch=0, checks=0):
    """Run a deck to completion; returns the list of per-step StepInfo."""
    drv = Driver(deck_text, mode, max_iters_cap, log_path, cap_after_switch, checks)
    steps = []
    try:
        while True:
            info = drv.step()
            if info is None:
                break
            steps.append(info)
            if info.complete:
                break
    finally:
        drv.close()
    return steps


class Batch:
    """Many independent single-chunk CG problems solved together on the GPU
    (tea_gb300_batch_* in include/tealeaf_gb300.h).  sizes: list of
    (x_cells, y_cells)."""

    def __init__(self, sizes, prec="jac_diag", coefficient=1,
                 extent=(0.0, 10.0, 0.0, 10.0)):
        L = load()
        self.sizes = [(int(x), int(y)) for x, y in sizes]
        xs = np.array([x for x, _ in self.sizes], dtype=np.int32)
        ys = np.array([y for _, y in self.sizes], dtype=np.int32)
        self.steps = 0
        if L.tea_gb300_batch_create(len(self.sizes), _pi(xs), _pi(ys), *map(float, extent),
                                    PREC[prec] if isinstance(prec, str) else int(prec),
                                    int(coefficient)) != 0:
            check()
            raise TeaError("batch_create failed")

    def set_fields(self, i, density, energy):
        x, y = self.sizes[i]
        d = np.ascontiguousarray(density, dtype=np.float64)
        e = np.ascontiguousarray(energy, dtype=np.float64)
        assert d.shape == (y, x) and e.shape == (y, x)
        if load().tea_gb300_batch_set_fields(i, _pd(d), _pd(e)) != 0:
            check()
            raise TeaError("batch_set_fields failed")

    def run(self, steps, dt, eps, max_iters):
        st = BatchStats()
        if load().tea_gb300_batch_run(int(steps), float(dt), float(eps), int(max_iters),
                                      C.byref(st)) != 0:
            check()
            raise TeaError("batch_run failed")
        self.steps = int(steps)
        return st

    def summary(self, i):
        out = np.zeros(4)
        if load().tea_gb300_batch_summary(i, _pd(out)) != 0:
            check()
            raise TeaError("batch_summary failed")
        return tuple(out)

    def iterations(self, i):
        out = np.zeros(self.steps, dtype=np.int32)
        if load().tea_gb300_batch_iterations(i, _pi(out), self.steps) != 0:
            check()
            raise TeaError("batch_iterations failed")
        return [int(v) for v in out]

    def read(self, i, name):
        x, y = self.sizes[i]
        out = np.zeros((y, x))
        if load().tea_gb300_batch_read_field(i, FIELD[name], _pd(out)) != 0:
            check()
            raise TeaError("batch_read_field failed")
        return out

    def launch(self):
        l = BatchLaunch()
        if load().tea_gb300_batch_get_launch(C.byref(l)) != 0:
            check()
        return l.as_dict()

    def set_launch(self, blocks_per_sm, graph_iterations=16, supertiles_per_unit=1,
                   persistent=0):
        l = BatchLaunch(int(blocks_per_sm), int(graph_iterations), int(supertiles_per_unit),
                        int(persistent))
        if load().tea_gb300_batch_set_launch(C.byref(l)) != 0:
            check()
            raise TeaError("batch_set_launch failed")

    def autotune(self):
        l = BatchLaunch()
        if load().tea_gb300_batch_autotune(C.byref(l)) != 0:
            check()
            raise TeaError("batch_autotune failed")
        return l.as_dict()

    def free(self):
        load().tea_gb300_batch_free()


def _devptr(t):
    """Device address of a CUDA tensor (or an int address), or None."""
    if t is None:
        return None
    return C.c_void_p(t if isinstance(t, int) else t.data_ptr())


class Adjoint:
    """The time-stepped solve and its adjoint w.r.t. log-density
    (tea_gb300_adjoint_* in include/tealeaf_gb300.h).  Field arguments are
    contiguous float64 CUDA tensors of shape (y_cells, x_cells)."""

    def __init__(self, x_cells, y_cells, coefficient=1, prec="jac_diag",
                 extent=(0.0, 10.0, 0.0, 10.0)):
        self.shape = (int(y_cells), int(x_cells))
        if load().tea_gb300_adjoint_create(int(x_cells), int(y_cells), *map(float, extent),
                                           int(coefficient),
                                           PREC[prec] if isinstance(prec, str) else int(prec)) != 0:
            check()
            raise TeaError("adjoint_create failed")

    @staticmethod
    def config(steps, dt=0.004, eps=1e-12, max_iters=10000, checkpoint_every=4):
        return AdjointConfig(int(steps), float(dt), float(eps), int(max_iters),
                             int(checkpoint_every))

    def forward(self, density, energy0, u_obs=None, u_final=None, cfg=None):
        """Runs the forward model; returns (loss or None, AdjointStats)."""
        for t in (density, energy0, u_obs, u_final):
            if t is not None and not isinstance(t, int):
                assert t.is_cuda and t.is_contiguous() and tuple(t.shape) == self.shape
        loss = C.c_double()
        st = AdjointStats()
        if load().tea_gb300_adjoint_forward(_devptr(density), _devptr(energy0), _devptr(u_obs),
                                            C.byref(cfg), C.byref(loss), _devptr(u_final),
                                            C.byref(st)) != 0:
            check()
            raise TeaError("adjoint_forward failed")
        return (loss.value if u_obs is not None else None), st

    def backward(self, grad_out):
        """d loss / d log(density) of the last forward pass into grad_out."""
        st = AdjointStats()
        if load().tea_gb300_adjoint_backward(_devptr(grad_out), C.byref(st)) != 0:
            check()
            raise TeaError("adjoint_backward failed")
        return st

    def free(self):
        load().tea_gb300_adjoint_free()
