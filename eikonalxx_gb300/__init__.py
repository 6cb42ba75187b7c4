"""eikonalxx_gb300 -- GB300-native level-set fast-sweeping eikonal solver.

Python binding of the C ABI in include/eikx/eikx_c.h (libeikx.so, built in-tree by
eikonalxx_gb300/build.py).  The solve runs on the GPU through the native library;
there is no CPU fallback: importing the binding without the built library raises.

The objects mirror the reference's (uofuseismo/eikonalxx) solver workflow:
Solver3D.initialize(options, geometry) -> setVelocityModel -> setSource -> solve ->
getTravelTimeField, with many sources solved in one batched launch (``solve_batch``).
"""
import ctypes
import os
from dataclasses import dataclass, field

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libeikx.so")

EIKX_OK = 0
EIKX_ERR_INVALID = -1
EIKX_ERR_STATE = -2
EIKX_ERR_CUDA = -3
EIKX_ERR_TIMEOUT = -4
EIKX_ERR_ALLOC = -5
EIKX_ERR_UNSUPPORTED = -6
F32, F64 = 0, 1
HOST, DEVICE = 0, 1
NATURAL, TRANSPOSED = 0, 1

# every symbol include/eikx/eikx_c.h declares
EXPORTED = [
    "eikx_options_default", "eikx_create", "eikx_destroy", "eikx_last_error", "eikx_get_stats",
    "eikx_set_grid3d", "eikx_set_slowness3d", "eikx_set_nodal_velocity3d", "eikx_get_slowness3d",
    "eikx_solve3d", "eikx_set_grid2d", "eikx_set_slowness2d", "eikx_set_nodal_velocity2d",
    "eikx_solve2d", "eikx_graph3d_tables", "eikx_levels2d", "eikx_analytic3d", "eikx_analytic2d",
    "eikx_solve3d_noalloc", "eikx_solve3d_batch", "eikx_autotune3d", "eikx_tuning_save", "eikx_tuning_load",
    "eikx_gradient3d", "eikx_gradient2d", "eikx_station_times3d", "eikx_station_times2d", "eikx_solve3d_warm",
    "eikx_ray_options_default", "eikx_trace_rays2d",
    "eikx_warmnet_create", "eikx_warmnet_destroy", "eikx_warmnet_num_params", "eikx_warmnet_get_params",
    "eikx_warmnet_set_params", "eikx_warmnet_train_step", "eikx_warmnet_gradients", "eikx_warmnet_predict",
    "eikx_warmnet_profile_step", "eikx_warmnet_set_test_hooks", "eikx_selftest_operator3d",
]
CELL_SLOWNESS, NODAL_VELOCITY = 0, 1


class EikxError(RuntimeError):
    """A failed C-ABI call; ``code`` is the eikx_status."""

    def __init__(self, code, msg):
        super().__init__(f"eikx error {code}: {msg}")
        self.code = code


class InvalidArgument(EikxError, ValueError):
    pass


class StateError(EikxError):
    pass


class TimeoutError_(EikxError):
    pass


class _Options(ctypes.Structure):
    _fields_ = [("n_sweeps", ctypes.c_int), ("tolerance", ctypes.c_double),
                ("factored_radius", ctypes.c_int), ("init_sweeps", ctypes.c_int),
                ("init_fp64", ctypes.c_int), ("spin_limit_log2", ctypes.c_int),
                ("test_drop_blocks", ctypes.c_int), ("profile_sweeps", ctypes.c_int),
                ("pair_fields", ctypes.c_int), ("sweep_kernel", ctypes.c_int),
                ("block_shape", ctypes.c_int), ("blocks_per_sm", ctypes.c_int),
                ("test_tag_margin", ctypes.c_int), ("near_fp64", ctypes.c_int), ("warm_gate", ctypes.c_int),
                ("max_in_flight", ctypes.c_int), ("reserved", ctypes.c_int)]


class _Stats(ctypes.Structure):
    _fields_ = [("n_fields", ctypes.c_int), ("iterations_max", ctypes.c_int),
                ("iterations_min", ctypes.c_int), ("sweeps_launched", ctypes.c_int),
                ("kernel_launches", ctypes.c_int), ("residual_last", ctypes.c_double),
                ("device_ms", ctypes.c_double), ("sweep_ms", ctypes.c_double), ("reset_nodes", ctypes.c_longlong),
                ("refine_node_updates", ctypes.c_longlong)]


class _RayOptions(ctypes.Structure):
    _fields_ = [("n_radii", ctypes.c_int), ("radius", ctypes.c_int * 16), ("scale", ctypes.c_double * 16),
                ("max_steps", ctypes.c_int), ("reserved", ctypes.c_int)]


class _RaySeg(ctypes.Structure):
    _fields_ = [("x0", ctypes.c_double), ("z0", ctypes.c_double), ("x1", ctypes.c_double), ("z1", ctypes.c_double),
                ("slowness", ctypes.c_double), ("cell", ctypes.c_int), ("reserved", ctypes.c_int)]


class _NetConfig(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int), ("dx", ctypes.c_double),
                ("dy", ctypes.c_double), ("dz", ctypes.c_double), ("x0", ctypes.c_double), ("y0", ctypes.c_double),
                ("z0", ctypes.c_double), ("batch", ctypes.c_int), ("seed", ctypes.c_ulonglong)]


class _NetSample(ctypes.Structure):
    _fields_ = [("velocity", ctypes.c_void_p), ("travel_time", ctypes.c_void_p), ("x", ctypes.c_double),
                ("y", ctypes.c_double), ("z", ctypes.c_double)]


class _Src3(ctypes.Structure):
    _fields_ = [("x", ctypes.c_double), ("y", ctypes.c_double), ("z", ctypes.c_double)]


class _Src2(ctypes.Structure):
    _fields_ = [("x", ctypes.c_double), ("z", ctypes.c_double)]


class _Tuning(ctypes.Structure):
    _fields_ = [("sweep_kernel", ctypes.c_int), ("pair_fields", ctypes.c_int), ("block_shape", ctypes.c_int),
                ("blocks_per_sm", ctypes.c_int), ("ms_per_sweep", ctypes.c_double),
                ("default_ms_per_sweep", ctypes.c_double), ("candidates", ctypes.c_int)]


class _Model3(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double),
                ("x0", ctypes.c_double), ("y0", ctypes.c_double), ("z0", ctypes.c_double),
                ("model", ctypes.c_void_p), ("model_kind", ctypes.c_int), ("dtype", ctypes.c_int),
                ("ordering", ctypes.c_int), ("where", ctypes.c_int), ("n_src", ctypes.c_int),
                ("src", ctypes.POINTER(_Src3)), ("t_out", ctypes.c_void_p), ("t_where", ctypes.c_int)]


_lib = None


def load(path=None):
    """Load libeikx.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError(f"{p} is missing: build it with `python eikonalxx_gb300/build.py` "
                          "(the solver has no CPU fallback)")
    lib = ctypes.CDLL(p)
    c_int, c_double, vp = ctypes.c_int, ctypes.c_double, ctypes.c_void_p
    ip = ctypes.POINTER(ctypes.c_int)
    lib.eikx_options_default.argtypes = [ctypes.POINTER(_Options)]
    lib.eikx_options_default.restype = None
    lib.eikx_create.argtypes = [ctypes.POINTER(vp), c_int]
    lib.eikx_destroy.argtypes = [vp]
    lib.eikx_last_error.restype = ctypes.c_char_p
    lib.eikx_get_stats.argtypes = [vp, ctypes.POINTER(_Stats)]
    lib.eikx_set_grid3d.argtypes = [vp, c_int, c_int, c_int] + [c_double] * 6
    lib.eikx_set_slowness3d.argtypes = [vp, vp, c_int, c_int, c_int]
    lib.eikx_set_nodal_velocity3d.argtypes = [vp, vp, c_int, c_int, c_int]
    lib.eikx_get_slowness3d.argtypes = [vp, vp, c_int]
    lib.eikx_solve3d.argtypes = [vp, ctypes.POINTER(_Src3), c_int, ctypes.POINTER(_Options), c_int, vp, c_int]
    lib.eikx_set_grid2d.argtypes = [vp, c_int, c_int] + [c_double] * 4
    lib.eikx_set_slowness2d.argtypes = [vp, vp, c_int, c_int, c_int]
    lib.eikx_set_nodal_velocity2d.argtypes = [vp, vp, c_int, c_int, c_int]
    lib.eikx_solve2d.argtypes = [vp, ctypes.POINTER(_Src2), c_int, ctypes.POINTER(_Options), c_int, vp, c_int]
    lib.eikx_graph3d_tables.argtypes = [c_int, c_int, c_int, c_int, ip, ip, ip, ip, ip, ip, ip]
    lib.eikx_levels2d.argtypes = [c_int, c_int, c_int, ip, ip, ip]
    lib.eikx_analytic3d.argtypes = [vp, ctypes.POINTER(_Src3), c_double, c_double, vp, c_int]
    lib.eikx_analytic2d.argtypes = [vp, ctypes.POINTER(_Src2), c_double, c_double, vp, c_int]
    lib.eikx_solve3d_batch.argtypes = [vp, ctypes.POINTER(_Model3), c_int, ctypes.POINTER(_Options), c_int]
    lib.eikx_autotune3d.argtypes = [vp, ctypes.POINTER(_Src3), c_int, c_int, ctypes.POINTER(_Tuning)]
    lib.eikx_solve3d_warm.argtypes = [vp, ctypes.POINTER(_Src3), c_int, ctypes.POINTER(_Options), c_int, vp, c_int,
                                      c_double, vp, c_int]
    lib.eikx_gradient3d.argtypes = [vp, c_int, vp, c_int]
    lib.eikx_gradient2d.argtypes = [vp, c_int, vp, c_int]
    lib.eikx_station_times3d.argtypes = [vp, c_int, ctypes.POINTER(_Src3), c_int, ctypes.POINTER(c_double)]
    lib.eikx_station_times2d.argtypes = [vp, c_int, ctypes.POINTER(_Src2), c_int, ctypes.POINTER(c_double)]
    dp = ctypes.POINTER(c_double)
    fp = ctypes.POINTER(ctypes.c_float)
    sp = ctypes.POINTER(_NetSample)
    lib.eikx_warmnet_create.argtypes = [c_int, ctypes.POINTER(_NetConfig), ctypes.POINTER(vp)]
    lib.eikx_warmnet_destroy.argtypes = [vp]
    lib.eikx_warmnet_num_params.argtypes = [vp, ctypes.POINTER(ctypes.c_longlong)]
    lib.eikx_warmnet_get_params.argtypes = [vp, fp]
    lib.eikx_warmnet_set_params.argtypes = [vp, fp]
    lib.eikx_warmnet_train_step.argtypes = [vp, sp, c_int, ctypes.c_float, dp]
    lib.eikx_warmnet_gradients.argtypes = [vp, sp, c_int, fp, dp]
    lib.eikx_warmnet_predict.argtypes = [vp, sp, c_int, c_double, vp, c_int, dp]
    lib.eikx_warmnet_profile_step.argtypes = [vp, sp, c_int, ctypes.c_float, dp, dp]
    lib.eikx_warmnet_set_test_hooks.argtypes = [vp, c_int, c_int]
    lib.eikx_selftest_operator3d.argtypes = [c_int, c_int, ctypes.c_longlong, ctypes.c_ulonglong,
                                             ctypes.POINTER(ctypes.c_longlong)]
    lib.eikx_tuning_save.argtypes = [vp, ctypes.c_char_p]
    lib.eikx_tuning_load.argtypes = [vp, ctypes.c_char_p]
    for name in EXPORTED:
        if name not in ("eikx_options_default", "eikx_last_error", "eikx_levels2d", "eikx_graph3d_tables",
                        "eikx_ray_options_default"):
            getattr(lib, name).restype = c_int
    lib.eikx_graph3d_tables.restype = c_int
    lib.eikx_levels2d.restype = c_int
    _lib = lib
    return lib


def _check(rc):
    if rc == EIKX_OK:
        return
    msg = load().eikx_last_error().decode()
    if rc == EIKX_ERR_INVALID:
        raise InvalidArgument(rc, msg)
    if rc == EIKX_ERR_STATE:
        raise StateError(rc, msg)
    if rc == EIKX_ERR_TIMEOUT:
        raise TimeoutError_(rc, msg)
    raise EikxError(rc, msg)


@dataclass
class Options:
    """SolverOptions (include/eikonalxx/solverOptions.hpp) plus the GPU knobs."""
    n_sweeps: int = 5
    tolerance: float = 1e-5
    factored_radius: int = 3
    init_sweeps: bool = True
    init_fp64: bool = True
    spin_limit_log2: int = 22
    test_drop_blocks: int = 0   # test hook only (see eikx_options.test_drop_blocks)
    profile_sweeps: bool = False  # time each sweep kernel with CUDA events (no graph)
    pair_fields: bool = False     # two fields per GPU lane for FP32 uniform batches
    sweep_kernel: int = 0         # 3D: 0 = tuned or chunk-step, 1 = node-step, 2 = chunk-step
    block_shape: int = 0          # 3D chunk-step warp block: 0 = tuned or 8x4, 1 = 8x4, 2 = 4x8, 3 = 16x2
    blocks_per_sm: int = 0        # persistent grid: 0 = as many as fit (or tuned)
    test_tag_margin: int = 0      # test hook only (see eikx_options.test_tag_margin)
    near_fp64: bool = False       # 3D FP32: factored (near-source) updates in FP64
    warm_gate: int = 0            # solve3d_warm residual gate: 0 one-sided, 1 two-sided
    max_in_flight: int = 0        # solve3d: > 0 = a stream of the sources through this many slots

    def _c(self):
        o = _Options()
        o.n_sweeps = int(self.n_sweeps)
        o.tolerance = float(self.tolerance)
        o.factored_radius = int(self.factored_radius)
        o.init_sweeps = int(bool(self.init_sweeps))
        o.init_fp64 = int(bool(self.init_fp64))
        o.spin_limit_log2 = int(self.spin_limit_log2)
        o.test_drop_blocks = int(self.test_drop_blocks)
        o.profile_sweeps = int(bool(self.profile_sweeps))
        o.pair_fields = int(bool(self.pair_fields))
        o.sweep_kernel = int(self.sweep_kernel)
        o.block_shape = int(self.block_shape)
        o.blocks_per_sm = int(self.blocks_per_sm)
        o.test_tag_margin = int(self.test_tag_margin)
        o.near_fp64 = int(bool(self.near_fp64))
        o.warm_gate = int(self.warm_gate)
        o.max_in_flight = int(self.max_in_flight)
        return o


def _ptr(a):
    """(pointer, where) of a numpy array or a CUDA torch tensor."""
    if isinstance(a, np.ndarray):
        if not a.flags["C_CONTIGUOUS"]:
            raise ValueError("arrays must be C-contiguous")
        return ctypes.c_void_p(a.ctypes.data), HOST
    if hasattr(a, "data_ptr") and hasattr(a, "is_cuda"):
        if not a.is_contiguous():
            raise ValueError("tensors must be contiguous")
        return ctypes.c_void_p(a.data_ptr()), (DEVICE if a.is_cuda else HOST)
    raise TypeError("expected a numpy array or a torch tensor")


def _dtype_code(a):
    dt = str(a.dtype)
    if dt in ("float32", "torch.float32"):
        return F32
    if dt in ("float64", "torch.float64"):
        return F64
    raise TypeError(f"unsupported dtype {dt}")


class Context:
    """One GPU, its stream, buffers and cached sweep-schedule graphs (eikx_ctx)."""

    def __init__(self, device=0):
        lib = load()
        h = ctypes.c_void_p()
        _check(lib.eikx_create(ctypes.byref(h), int(device)))
        self._h = h
        self._lib = lib
        self.grid3 = None
        self.grid2 = None

    def close(self):
        if getattr(self, "_h", None):
            self._lib.eikx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- 3D ---------------------------------------------------------------
    def set_grid3d(self, nx, ny, nz, dx, dy, dz, x0=0.0, y0=0.0, z0=0.0):
        _check(self._lib.eikx_set_grid3d(self._h, nx, ny, nz, dx, dy, dz, x0, y0, z0))
        self.grid3 = (nx, ny, nz, dx, dy, dz, x0, y0, z0)

    def set_slowness3d(self, s, ordering=NATURAL):
        p, where = _ptr(s)
        _check(self._lib.eikx_set_slowness3d(self._h, p, _dtype_code(s), ordering, where))

    def set_nodal_velocity3d(self, v, ordering=NATURAL):
        p, where = _ptr(v)
        _check(self._lib.eikx_set_nodal_velocity3d(self._h, p, _dtype_code(v), ordering, where))

    def get_slowness3d(self, dtype=np.float64):
        nx, ny, nz = self.grid3[:3]
        out = np.empty((nx - 1) * (ny - 1) * (nz - 1), dtype=dtype)
        _check(self._lib.eikx_get_slowness3d(self._h, ctypes.c_void_p(out.ctypes.data), _dtype_code(out)))
        return out

    def solve3d(self, sources, options=None, precision=F32, out=None):
        """Solve one field per source; returns (n_src, nz, ny, nx) (numpy, or `out`)."""
        src = np.atleast_2d(np.asarray(sources, dtype=np.float64))
        n = src.shape[0]
        arr = (_Src3 * n)(*[_Src3(*map(float, s)) for s in src])
        nx, ny, nz = self.grid3[:3]
        if out is None:
            out = np.empty((n, nz, ny, nx), dtype=np.float32 if precision == F32 else np.float64)
        p, where = _ptr(out)
        o = (options or Options())._c()
        _check(self._lib.eikx_solve3d(self._h, arr, n, ctypes.byref(o), precision, p, where))
        return out

    def solve3d_warm(self, sources, t_init, options=None, precision=F32, gate_tol=1e-6, out=None):
        """Solve from initial fields `t_init` (n_src, nz, ny, nx): underestimated nodes are
        reset, then sweeps run to the tolerance without the initialisation pass."""
        src = np.atleast_2d(np.asarray(sources, dtype=np.float64))
        n = src.shape[0]
        arr = (_Src3 * n)(*[_Src3(*map(float, q)) for q in src])
        nx, ny, nz = self.grid3[:3]
        if out is None:
            out = np.empty((n, nz, ny, nx), dtype=np.float32 if precision == F32 else np.float64)
        ip, iwhere = _ptr(t_init)
        p, where = _ptr(out)
        o = (options or Options())._c()
        _check(self._lib.eikx_solve3d_warm(self._h, arr, n, ctypes.byref(o), precision, ip, iwhere, float(gate_tol),
                                           p, where))
        return out

    def gradient3d(self, field=0, precision=F32, out=None):
        """Travel-time gradient of field `field` of the last 3D solve: (nz, ny, nx, 3)."""
        if self.grid3 is None:                       # no solve yet: the library reports it
            _check(self._lib.eikx_gradient3d(self._h, int(field), None, HOST))
        nx, ny, nz = self.grid3[:3]
        if out is None:
            out = np.empty((nz, ny, nx, 3), dtype=np.float32 if precision == F32 else np.float64)
        p, where = _ptr(out)
        _check(self._lib.eikx_gradient3d(self._h, int(field), p, where))
        return out

    def gradient2d(self, field=0, precision=F64, out=None):
        """Travel-time gradient of field `field` of the last 2D solve: (nz, nx, 2)."""
        if self.grid2 is None:
            _check(self._lib.eikx_gradient2d(self._h, int(field), None, HOST))
        nx, nz = self.grid2[:2]
        if out is None:
            out = np.empty((nz, nx, 2), dtype=np.float32 if precision == F32 else np.float64)
        p, where = _ptr(out)
        _check(self._lib.eikx_gradient2d(self._h, int(field), p, where))
        return out

    def station_times3d(self, stations, field=0):
        st = np.atleast_2d(np.asarray(stations, dtype=np.float64))
        arr = (_Src3 * len(st))(*[_Src3(*map(float, q)) for q in st])
        out = np.empty(len(st), dtype=np.float64)
        _check(self._lib.eikx_station_times3d(self._h, int(field), arr, len(st),
                                              out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return out

    def station_times2d(self, stations, field=0):
        st = np.atleast_2d(np.asarray(stations, dtype=np.float64))
        arr = (_Src2 * len(st))(*[_Src2(float(q[0]), float(q[1])) for q in st])
        out = np.empty(len(st), dtype=np.float64)
        _check(self._lib.eikx_station_times2d(self._h, int(field), arr, len(st),
                                              out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return out

    def trace_rays2d(self, gradient, slowness, source, stations, radius_scale=None, max_steps=0, capacity=None,
                     grid=None):
        """Ray::GradientTracer2D::trace: rays from the stations to the source down a gradient
        field (nz, nx, 2) with cell slowness ((nz-1)*(nx-1), FP64).  grid = (nx, nz, dx, dz,
        x0, z0), default the context's 2D grid; radius_scale = [(radius, scale), ...], default
        the reference's.  Returns (paths, counts): paths[i] is an (n_i, 6) array of (x0, z0, x1,
        z1, slowness, cell) or None when counts[i] < 0 (-1 no convergence, -2 capacity, -3 left
        the grid)."""
        nx, nz, dx, dz, x0, z0 = grid if grid is not None else self.grid2
        g = np.ascontiguousarray(gradient)
        if g.dtype not in (np.float32, np.float64) or g.size != 2 * nx * nz:
            raise InvalidArgument(-2, "gradient must hold nz * nx * 2 FP32 or FP64 values")
        s = np.ascontiguousarray(slowness, dtype=np.float64).ravel()
        st = np.ascontiguousarray(np.atleast_2d(np.asarray(stations, dtype=np.float64)))
        n = len(st)
        opt = _RayOptions()
        self._lib.eikx_ray_options_default(ctypes.byref(opt))
        if radius_scale is not None:
            opt.n_radii = len(radius_scale)
            for k, (r, sc) in enumerate(radius_scale):
                opt.radius[k] = int(r)
                opt.scale[k] = float(sc)
        opt.max_steps = int(max_steps)
        cap = int(capacity) if capacity else 4 * (nx + nz) + 16
        segs = (_RaySeg * (n * cap))()
        counts = np.zeros(n, dtype=np.int32)
        _check(self._lib.eikx_trace_rays2d(
            self._h, nx, nz, ctypes.c_double(dx), ctypes.c_double(dz), ctypes.c_double(x0), ctypes.c_double(z0),
            ctypes.c_void_p(g.ctypes.data), F64 if g.dtype == np.float64 else F32,
            s.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.c_double(float(source[0])),
            ctypes.c_double(float(source[1])), st.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), n,
            ctypes.byref(opt), cap, segs, counts.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))
        raw = np.frombuffer(segs, dtype=np.dtype([("x0", "f8"), ("z0", "f8"), ("x1", "f8"), ("z1", "f8"),
                                                  ("slowness", "f8"), ("cell", "i4"), ("reserved", "i4")]))
        paths = []
        for i in range(n):
            if counts[i] <= 0:
                paths.append(None)
                continue
            r = raw[i * cap:i * cap + counts[i]]
            paths.append(np.column_stack([r["x0"], r["z0"], r["x1"], r["z1"], r["slowness"], r["cell"]]))
        return paths, counts

    def autotune3d(self, sources, precision=F32):
        """Time the kernel variants, warp-block shapes and grid sizes on this model and these
        sources; later solves of the same grid class with default options use the fastest.
        Returns the choice as a dict."""
        src = np.atleast_2d(np.asarray(sources, dtype=np.float64))
        arr = (_Src3 * len(src))(*[_Src3(*map(float, q)) for q in src])
        t = _Tuning()
        _check(self._lib.eikx_autotune3d(self._h, arr, len(src), precision, ctypes.byref(t)))
        return {k: getattr(t, k) for k, _ in _Tuning._fields_}

    def save_tuning(self, path):
        _check(self._lib.eikx_tuning_save(self._h, os.fsencode(path)))

    def load_tuning(self, path):
        _check(self._lib.eikx_tuning_load(self._h, os.fsencode(path)))

    def solve3d_batch(self, models, options=None, precision=F32):
        """Solve many models, each with its own sources, in one schedule.

        `models` is a sequence of dicts with keys ``grid`` = (nx, ny, nz, dx, dy, dz[, x0,
        y0, z0]), ``model`` (cell slowness of (nz-1, ny-1, nx-1) values or, with
        ``nodal=True``, nodal velocity of (nz, ny, nx) values; numpy or torch, host or
        CUDA), ``sources`` (sequence of (x, y, z)) and optionally ``out`` (n_src, nz, ny,
        nx). Returns the list of output arrays, one per model."""
        n = len(models)
        arr = (_Model3 * n)()
        keep, outs = [], []
        for i, m in enumerate(models):
            g = tuple(m["grid"]) + (0.0,) * (9 - len(m["grid"]))
            nx, ny, nz = (int(v) for v in g[:3])
            src = np.atleast_2d(np.asarray(m["sources"], dtype=np.float64))
            sarr = (_Src3 * len(src))(*[_Src3(*map(float, q)) for q in src])
            out = m.get("out")
            if out is None:
                out = np.empty((len(src), nz, ny, nx), dtype=np.float32 if precision == F32 else np.float64)
            mp, mwhere = _ptr(m["model"])
            op, owhere = _ptr(out)
            arr[i] = _Model3(nx, ny, nz, *map(float, g[3:9]), mp,
                             NODAL_VELOCITY if m.get("nodal") else CELL_SLOWNESS, _dtype_code(m["model"]),
                             int(m.get("ordering", NATURAL)), mwhere, len(src), sarr, op, owhere)
            keep.append(sarr)
            outs.append(out)
        o = (options or Options())._c()
        _check(self._lib.eikx_solve3d_batch(self._h, arr, n, ctypes.byref(o), precision))
        return outs

    # ---- 2D ---------------------------------------------------------------
    def set_grid2d(self, nx, nz, dx, dz, x0=0.0, z0=0.0):
        _check(self._lib.eikx_set_grid2d(self._h, nx, nz, dx, dz, x0, z0))
        self.grid2 = (nx, nz, dx, dz, x0, z0)

    def set_slowness2d(self, s, ordering=NATURAL):
        p, where = _ptr(s)
        _check(self._lib.eikx_set_slowness2d(self._h, p, _dtype_code(s), ordering, where))

    def set_nodal_velocity2d(self, v, ordering=NATURAL):
        p, where = _ptr(v)
        _check(self._lib.eikx_set_nodal_velocity2d(self._h, p, _dtype_code(v), ordering, where))

    def solve2d(self, sources, options=None, precision=F64, out=None):
        """Solve one field per (x, z) source; returns (n_src, nz, nx)."""
        src = np.atleast_2d(np.asarray(sources, dtype=np.float64))
        n = src.shape[0]
        arr = (_Src2 * n)(*[_Src2(float(s[0]), float(s[1])) for s in src])
        nx, nz = self.grid2[:2]
        if out is None:
            out = np.empty((n, nz, nx), dtype=np.float32 if precision == F32 else np.float64)
        p, where = _ptr(out)
        o = (options or Options())._c()
        _check(self._lib.eikx_solve2d(self._h, arr, n, ctypes.byref(o), precision, p, where))
        return out

    # ---- analytic (FP64, GPU) -----------------------------------------------
    def analytic3d(self, source, v_top, v_bottom):
        nx, ny, nz = self.grid3[:3]
        out = np.empty((nz, ny, nx), dtype=np.float64)
        s = _Src3(*map(float, source))
        _check(self._lib.eikx_analytic3d(self._h, ctypes.byref(s), v_top, v_bottom,
                                         ctypes.c_void_p(out.ctypes.data), HOST))
        return out

    def analytic2d(self, source, v_top, v_bottom):
        nx, nz = self.grid2[:2]
        out = np.empty((nz, nx), dtype=np.float64)
        s = _Src2(float(source[0]), float(source[1]))
        _check(self._lib.eikx_analytic2d(self._h, ctypes.byref(s), v_top, v_bottom,
                                         ctypes.c_void_p(out.ctypes.data), HOST))
        return out

    def stats(self):
        s = _Stats()
        _check(self._lib.eikx_get_stats(self._h, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in _Stats._fields_}


def selftest_operator3d(n, seed=1, precision=F32, device=0):
    """Run the device self-test of the 3D sweep's operator shortcuts on n seeded stencils at
    their edges; returns counts: evaluated, mismatches (0 = exact), results equal to t0,
    stencils whose t0 is the operator's own value."""
    lib = load()
    out = (ctypes.c_longlong * 4)()
    _check(lib.eikx_selftest_operator3d(device, precision, n, seed, out))
    return dict(zip(("evaluated", "mismatches", "shortcut_t0", "t0_is_operator"), list(out)))


def graph3d_tables(sweep, nx, ny, nz):
    """Graph3D<Sweep(sweep+1)> tables (host): dict of numpy int32 arrays."""
    lib = load()
    n = nx * ny * nz
    ls = np.zeros(nx + ny + nz - 1, np.int32)
    arrs = [np.zeros(n, np.int32) for _ in range(5)]
    mx = ctypes.c_int(0)
    P = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    nl = lib.eikx_graph3d_tables(sweep, nx, ny, nz, P(ls), *[P(a) for a in arrs], ctypes.byref(mx))
    if nl < 0:
        _check(nl)
    return {"n_levels": nl, "level_start": ls, "node_to_index": arrs[0], "to_x": arrs[1],
            "to_y": arrs[2], "to_z": arrs[3], "index_to_level": arrs[4], "max_level_size": mx.value}


def levels2d(sweep, nx, nz):
    """2D level-set visiting order (host): (level_start, ix, iz)."""
    lib = load()
    ls = np.zeros(nx + nz, np.int32)
    ix = np.zeros(nx * nz, np.int32)
    iz = np.zeros(nx * nz, np.int32)
    P = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    nl = lib.eikx_levels2d(sweep, nx, nz, P(ls), P(ix), P(iz))
    if nl < 0:
        _check(nl)
    return ls, ix, iz
