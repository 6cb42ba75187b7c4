"""ORACLE -- test infrastructure only.

ctypes front-ends of the CPU checkers: the project's restatement of the reference's
algorithm (libeikx_oracle.so, eikx_oracle.cpp) and, where it was built, the
reference's own code (libeikx_ref.so, ref_driver.cpp).  Imported only by tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline legs; the solver never uses it.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_d = ctypes.c_double
_P = lambda a: ctypes.c_void_p(a.ctypes.data)


def _load(path):
    return ctypes.CDLL(path)


class Oracle:
    """The project's CPU restatement (bit-identical to the reference's sweep)."""

    def __init__(self):
        self.lib = _load(_build.build_oracle())
        self.lib.oracle_sweep3d_f32.restype = ctypes.c_double
        self.lib.oracle_sweep3d_f64.restype = ctypes.c_double
        self.lib.oracle_hypot.restype = ctypes.c_double

    def solve3d(self, slow, grid, src_cell, src_off, n_sweeps=2, radius=3, tol=-1.0, init_fp64=True,
                init_sweeps=True, residuals=False, near_fp64=False):
        nx, ny, nz, dx, dy, dz = grid
        dt = slow.dtype
        tt = np.zeros(nx * ny * nz, dt)
        res = np.zeros(max(1, 8 * n_sweeps), np.float64)
        it = ctypes.c_int(0)
        f = self.lib.oracle_solve3d_f64 if dt == np.float64 else self.lib.oracle_solve3d_f32
        self.lib.oracle_set_near_fp64(int(bool(near_fp64)))
        try:
            f(nx, ny, nz, _d(dx), _d(dy), _d(dz), int(src_cell[0]), int(src_cell[1]), int(src_cell[2]),
              _d(src_off[0]), _d(src_off[1]), _d(src_off[2]), _P(np.ascontiguousarray(slow)), n_sweeps, radius,
              _d(tol), int(init_fp64), int(init_sweeps), _P(tt), _P(res), ctypes.byref(it))
        finally:
            self.lib.oracle_set_near_fp64(0)
        tt = tt.reshape(nz, ny, nx)
        return (tt, res[:8 * it.value].reshape(-1, 8), it.value) if residuals else tt

    def solve2d(self, slow, grid, src_cell, src_off, n_sweeps=2, radius=3, tol=-1.0, init_fp64=True,
                init_sweeps=True, hypot_mode=1, residuals=False):
        nx, nz, dx, dz = grid
        dt = slow.dtype
        self.lib.oracle_set_hypot_mode(int(hypot_mode))
        tt = np.zeros(nx * nz, dt)
        res = np.zeros(max(1, 4 * n_sweeps), np.float64)
        it = ctypes.c_int(0)
        f = self.lib.oracle_solve2d_f64 if dt == np.float64 else self.lib.oracle_solve2d_f32
        f(nx, nz, _d(dx), _d(dz), int(src_cell[0]), int(src_cell[1]), _d(src_off[0]), _d(src_off[1]),
          _P(np.ascontiguousarray(slow)), n_sweeps, radius, _d(tol), int(init_fp64), int(init_sweeps),
          _P(tt), _P(res), ctypes.byref(it))
        tt = tt.reshape(nz, nx)
        return (tt, res[:4 * it.value].reshape(-1, 4), it.value) if residuals else tt

    def graph3d(self, sweep, nx, ny, nz):
        n = nx * ny * nz
        ls = np.zeros(nx + ny + nz - 1, np.int32)
        a = [np.zeros(n, np.int32) for _ in range(5)]
        mx = ctypes.c_int()
        nl = self.lib.oracle_graph3d(sweep, nx, ny, nz, _P(ls), *[_P(x) for x in a], ctypes.byref(mx))
        return {"n_levels": nl, "level_start": ls, "node_to_index": a[0], "to_x": a[1], "to_y": a[2],
                "to_z": a[3], "index_to_level": a[4], "max_level_size": mx.value}

    def linear_gradient3d(self, grid, src_off, v_top, v_bottom):
        nx, ny, nz, dx, dy, dz = grid
        t = np.zeros(nx * ny * nz)
        self.lib.oracle_linear_gradient3d(nx, ny, nz, _d(dx), _d(dy), _d(dz), _d(src_off[0]), _d(src_off[1]),
                                          _d(src_off[2]), _d(v_top), _d(v_bottom), _P(t))
        return t.reshape(nz, ny, nx)

    def linear_gradient2d(self, grid, src_off, v_top, v_bottom):
        nx, nz, dx, dz = grid
        t = np.zeros(nx * nz)
        self.lib.oracle_linear_gradient2d(nx, nz, _d(dx), _d(dz), _d(src_off[0]), _d(src_off[1]), _d(v_top),
                                          _d(v_bottom), _P(t))
        return t.reshape(nz, nx)

    def gradient3d(self, tt, grid, src_cell, src_off, slow0):
        """Central-difference gradient (nz, ny, nx, 3) of a solved field (src/gradient.hpp)."""
        nx, ny, nz, dx, dy, dz = grid
        tt = np.ascontiguousarray(tt)
        g = np.zeros(tt.size * 3, tt.dtype)
        f = self.lib.oracle_gradient3d_f64 if tt.dtype == np.float64 else self.lib.oracle_gradient3d_f32
        cv = ctypes.c_double if tt.dtype == np.float64 else ctypes.c_float
        f(nx, ny, nz, _d(dx), _d(dy), _d(dz), int(src_cell[0]), int(src_cell[1]), int(src_cell[2]),
          _d(src_off[0]), _d(src_off[1]), _d(src_off[2]), cv(slow0), _P(tt), _P(g))
        return g.reshape(nz, ny, nx, 3)

    def gradient2d(self, tt, grid, src_cell, src_off, slow0):
        nx, nz, dx, dz = grid
        tt = np.ascontiguousarray(tt)
        g = np.zeros(tt.size * 2, tt.dtype)
        f = self.lib.oracle_gradient2d_f64 if tt.dtype == np.float64 else self.lib.oracle_gradient2d_f32
        cv = ctypes.c_double if tt.dtype == np.float64 else ctypes.c_float
        f(nx, nz, _d(dx), _d(dz), int(src_cell[0]), int(src_cell[1]), _d(src_off[0]), _d(src_off[1]), cv(slow0),
          _P(tt), _P(g))
        return g.reshape(nz, nx, 2)

    def stations3d(self, tt, grid, src_cell, src_off, s_src, cells, offs):
        nx, ny, nz, dx, dy, dz = grid
        tt = np.ascontiguousarray(tt)
        cells = np.ascontiguousarray(cells, dtype=np.int32)
        offs = np.ascontiguousarray(offs, dtype=np.float64)
        out = np.zeros(len(cells), np.float64)
        self.lib.oracle_stations3d(0 if tt.dtype == np.float32 else 1, nx, ny, nz, _d(dx), _d(dy), _d(dz),
                                   int(src_cell[0]), int(src_cell[1]), int(src_cell[2]), _d(src_off[0]),
                                   _d(src_off[1]), _d(src_off[2]), _d(s_src), _P(tt), len(cells), _P(cells),
                                   _P(offs), _P(out))
        return out

    def trace_rays2d(self, grad, grid, origin, slow, source, stations, radii, scales, max_steps, capacity):
        """Ray::GradientTracer2D::trace: (segments [n][capacity][6], counts [n])."""
        nx, nz, dx, dz = grid
        grad = np.ascontiguousarray(grad)
        slow = np.ascontiguousarray(slow, dtype=np.float64)
        st = np.ascontiguousarray(stations, dtype=np.float64).reshape(-1, 2)
        n = len(st)
        seg = np.zeros((n, capacity, 6), np.float64)
        counts = np.zeros(n, np.int32)
        radii = np.ascontiguousarray(radii, dtype=np.int32)
        scales = np.ascontiguousarray(scales, dtype=np.float64)
        self.lib.oracle_trace_rays2d(0 if grad.dtype == np.float32 else 1, nx, nz, _d(dx), _d(dz), _d(origin[0]),
                                     _d(origin[1]), _P(grad), _P(slow), _d(source[0]), _d(source[1]), n, _P(st),
                                     len(radii), _P(radii), _P(scales), int(max_steps), int(capacity), _P(seg),
                                     _P(counts))
        return seg, counts

    def stations2d(self, tt, grid, src_cell, src_off, s_src, cells, offs):
        nx, nz, dx, dz = grid
        tt = np.ascontiguousarray(tt)
        cells = np.ascontiguousarray(cells, dtype=np.int32)
        offs = np.ascontiguousarray(offs, dtype=np.float64)
        out = np.zeros(len(cells), np.float64)
        self.lib.oracle_stations2d(0 if tt.dtype == np.float32 else 1, nx, nz, _d(dx), _d(dz), int(src_cell[0]),
                                   int(src_cell[1]), _d(src_off[0]), _d(src_off[1]), _d(s_src), _P(tt), len(cells),
                                   _P(cells), _P(offs), _P(out))
        return out

    def nodal_to_cell3d(self, v, nx, ny, nz, ordering=0):
        v = np.ascontiguousarray(v)
        s = np.zeros((nx - 1) * (ny - 1) * (nz - 1), v.dtype)
        f = self.lib.oracle_nodal_to_cell3d_f64 if v.dtype == np.float64 else self.lib.oracle_nodal_to_cell3d_f32
        f(nx, ny, nz, _P(v), ordering, _P(s))
        return s

    def nodal_to_cell2d(self, v, nx, nz, ordering=0):
        v = np.ascontiguousarray(v, dtype=np.float64)
        s = np.zeros((nx - 1) * (nz - 1))
        self.lib.oracle_nodal_to_cell2d_f64(nx, nz, _P(v), ordering, _P(s))
        return s


class ColdSolve3:
    """A cold-start FP32 3D solve run a bounded number of sweeps at a time, for the
    benchmark's CPU baselines: ``advance(n)`` runs up to n more sweeps of the schedule
    (initialisation, 8 source-limited sweeps, then refinement sweeps to the convergence
    rule) and returns True once the solve has ended.  ``sweeps`` counts the schedule sweeps
    run.  Run to the end, the field equals Oracle.solve3d's bit for bit."""

    def __init__(self, oracle, slow, grid, src_pos, n_sweeps, radius, tol, init_fp64=True):
        nx, ny, nz, dx, dy, dz = grid
        self._lib = oracle.lib
        self._slow = np.ascontiguousarray(slow, dtype=np.float32)
        self._grid = grid
        self._cell = [min(n - 2, int(p / d)) for p, n, d in zip(src_pos, (nx, ny, nz), (dx, dy, dz))]
        self._off = [float(p) for p in src_pos]
        self._args = (int(n_sweeps), int(radius), _d(tol), int(init_fp64))
        self.tt = np.empty(nx * ny * nz, np.float32)
        self._pos, self._quiet = ctypes.c_int(0), ctypes.c_int(0)
        self.done = False

    @property
    def sweeps(self):
        return self._pos.value

    def advance(self, n):
        nx, ny, nz, dx, dy, dz = self._grid
        c, o = self._cell, self._off
        n_sweeps, radius, tol, init_fp64 = self._args
        rc = self._lib.oracle_advance3d_f32(nx, ny, nz, _d(dx), _d(dy), _d(dz), c[0], c[1], c[2], _d(o[0]),
                                            _d(o[1]), _d(o[2]), _P(self._slow), n_sweeps, radius, tol, init_fp64,
                                            _P(self.tt), ctypes.byref(self._pos), ctypes.byref(self._quiet), int(n))
        self.done = bool(rc)
        return self.done


class Reference:
    """The reference's own sweep code (oracle/_ref); None-valued if not built."""

    def __init__(self):
        path = _build.build_ref()
        if path is None:
            raise FileNotFoundError("reference sources are not available here")
        self.lib = _load(path)

    def solve3d(self, slow, grid, src_cell, src_off, n_sweeps=2, radius=3, init_sweeps=True):
        nx, ny, nz, dx, dy, dz = grid
        tt = np.zeros(nx * ny * nz, slow.dtype)
        f = self.lib.ref_solve3d_f64 if slow.dtype == np.float64 else self.lib.ref_solve3d_f32
        rc = f(nx, ny, nz, _d(dx), _d(dy), _d(dz), int(src_cell[0]), int(src_cell[1]), int(src_cell[2]),
               _d(src_off[0]), _d(src_off[1]), _d(src_off[2]), _P(np.ascontiguousarray(slow)), n_sweeps,
               radius, int(init_sweeps), _P(tt))
        if rc != 0:
            raise RuntimeError("reference solve failed")
        return tt.reshape(nz, ny, nx)

    def solve2d(self, slow, grid, src_cell, src_off, n_sweeps=2, radius=3, init_sweeps=True):
        nx, nz, dx, dz = grid
        tt = np.zeros(nx * nz, slow.dtype)
        f = self.lib.ref_solve2d_f64 if slow.dtype == np.float64 else self.lib.ref_solve2d_f32
        rc = f(nx, nz, _d(dx), _d(dz), int(src_cell[0]), int(src_cell[1]), _d(src_off[0]), _d(src_off[1]),
               _P(np.ascontiguousarray(slow)), n_sweeps, radius, int(init_sweeps), _P(tt))
        if rc != 0:
            raise RuntimeError("reference solve failed")
        return tt.reshape(nz, nx)

    def trace_rays2d(self, grad, grid, origin, slow, source, stations, radii, scales, capacity):
        """The reference's own Ray::GradientTracer2D::trace: (segments [n][capacity][6], counts);
        a ray that does not reach the source has count 0 (an empty path)."""
        nx, nz, dx, dz = grid
        grad = np.ascontiguousarray(grad)
        slow = np.ascontiguousarray(slow, dtype=np.float64)
        st = np.ascontiguousarray(stations, dtype=np.float64).reshape(-1, 2)
        n = len(st)
        seg = np.zeros((n, capacity, 6), np.float64)
        counts = np.zeros(n, np.int32)
        radii = np.ascontiguousarray(radii, dtype=np.int32)
        scales = np.ascontiguousarray(scales, dtype=np.float64)
        rc = self.lib.ref_trace_rays2d(0 if grad.dtype == np.float32 else 1, nx, nz, _d(dx), _d(dz), _d(origin[0]),
                                       _d(origin[1]), _P(grad), _P(slow), _d(source[0]), _d(source[1]), n, _P(st),
                                       len(radii), _P(radii), _P(scales), int(capacity), _P(seg), _P(counts))
        if rc != 0:
            raise RuntimeError("reference ray tracing failed")
        return seg, counts

    def graph3d(self, sweep, nx, ny, nz):
        n = nx * ny * nz
        ls = np.zeros(nx + ny + nz - 1, np.int32)
        a = [np.zeros(n, np.int32) for _ in range(5)]
        mx = ctypes.c_int()
        nl = self.lib.ref_graph3d(sweep, nx, ny, nz, _P(ls), *[_P(x) for x in a], ctypes.byref(mx))
        return {"n_levels": nl, "level_start": ls, "node_to_index": a[0], "to_x": a[1], "to_y": a[2],
                "to_z": a[3], "index_to_level": a[4], "max_level_size": mx.value}


def source_cell(pos, origin, spacing, n):
    """Cell and offset of a source coordinate, as the reference's Source3D."""
    off = pos - origin
    return min(n - 2, int(off / spacing)), off
