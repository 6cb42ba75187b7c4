"""The reference's Python interface (module ``pyEikonalXX``, python/py*.cpp) over the GB300
solver: same class, property and method names, so scripts written for the reference run
unchanged after ``from eikonalxx_gb300 import pyEikonalXX``.

Value types (geometry, options, sources, stations, velocity models, ray points and
segments) are plain Python with the reference's validation.  Solver2D and Solver3D solve on
the GPU through the C ABI (``eikonalxx_gb300.Context``); the reference binds only Solver2D,
Solver3D is the same interface in 3D.  Fields come back as flat FP64 arrays in natural
order, as the reference's bindings return them (python/pySolver2d.cpp:100-160).
"""
import enum
import math

import numpy as np

from . import vtk as _vtk


class Ordering2D(enum.IntEnum):
    natural = 0
    zx = 0
    xz = 1


class Ordering3D(enum.IntEnum):
    natural = 0
    zyx = 0
    xyz = 1


class SolverAlgorithm(enum.IntEnum):
    level_set_method = 0
    fast_sweeping_method = 1


class Verbosity(enum.IntEnum):
    error = 0
    warning = 1
    info = 2
    debug = 3


def _positive(v, what):
    v = float(v)
    if not v > 0:
        raise ValueError(f"{what} = {v} must be positive")
    return v


def _at_least(n, lo, what):
    n = int(n)
    if n < lo:
        raise ValueError(f"{what} = {n} must be at least {lo}")
    return n


class Geometry2D:
    def __init__(self):
        self.clear()

    def clear(self):
        self._nx = self._nz = None
        self._dx = self._dz = None
        self.x0 = 0.0
        self.z0 = 0.0

    nx = property(lambda s: s._nx, lambda s, v: setattr(s, "_nx", _at_least(v, 3, "nx")))
    nz = property(lambda s: s._nz, lambda s, v: setattr(s, "_nz", _at_least(v, 3, "nz")))
    dx = property(lambda s: s._dx, lambda s, v: setattr(s, "_dx", _positive(v, "dx")))
    dz = property(lambda s: s._dz, lambda s, v: setattr(s, "_dz", _positive(v, "dz")))

    def __copy__(self):
        g = Geometry2D()
        g.__dict__.update(self.__dict__)
        return g

    def _complete(self):
        if None in (self._nx, self._nz, self._dx, self._dz):
            raise ValueError("geometry not fully set")


class Geometry3D:
    def __init__(self):
        self.clear()

    def clear(self):
        self._nx = self._ny = self._nz = None
        self._dx = self._dy = self._dz = None
        self.x0 = self.y0 = self.z0 = 0.0

    nx = property(lambda s: s._nx, lambda s, v: setattr(s, "_nx", _at_least(v, 3, "nx")))
    ny = property(lambda s: s._ny, lambda s, v: setattr(s, "_ny", _at_least(v, 3, "ny")))
    nz = property(lambda s: s._nz, lambda s, v: setattr(s, "_nz", _at_least(v, 3, "nz")))
    dx = property(lambda s: s._dx, lambda s, v: setattr(s, "_dx", _positive(v, "dx")))
    dy = property(lambda s: s._dy, lambda s, v: setattr(s, "_dy", _positive(v, "dy")))
    dz = property(lambda s: s._dz, lambda s, v: setattr(s, "_dz", _positive(v, "dz")))

    def __copy__(self):
        g = Geometry3D()
        g.__dict__.update(self.__dict__)
        return g

    def _complete(self):
        if None in (self._nx, self._ny, self._nz, self._dx, self._dy, self._dz):
            raise ValueError("geometry not fully set")


class SolverOptions:
    """Defaults as src/solverOptions.cpp:5-21."""

    def __init__(self):
        self.clear()

    def clear(self):
        self._sweeps = 5
        self.tolerance = 1.e-5
        self._radius = 3
        self.algorithm = SolverAlgorithm.level_set_method
        self.verbosity = Verbosity.error

    number_of_sweeps = property(lambda s: s._sweeps,
                                lambda s, v: setattr(s, "_sweeps", _at_least(v, 0, "number_of_sweeps")))
    factored_eikonal_equation_solver_radius = property(
        lambda s: s._radius, lambda s, v: setattr(s, "_radius", _at_least(v, 0, "factored radius")))

    def _options(self):
        from . import Options
        return Options(n_sweeps=self._sweeps, tolerance=float(self.tolerance), factored_radius=self._radius)


class _Point:
    """Source / station position: cell = min(nCell - 1, (x - x0) / dx), as
    Source3D::setLocationInX (src/source3d.cpp:161-185)."""

    def __init__(self):
        self._geometry = None
        self._loc = {}

    @property
    def geometry(self):
        if self._geometry is None:
            raise RuntimeError("geometry not set")
        return self._geometry

    @geometry.setter
    def geometry(self, g):
        g._complete()
        self._geometry = g.__copy__()
        self._loc = {}

    def _set(self, axis, v):
        g = self.geometry
        n, d, o = getattr(g, "n" + axis), getattr(g, "d" + axis), getattr(g, axis + "0")
        v = float(v)
        if not (o <= v <= o + (n - 1) * d):
            raise ValueError(f"{axis} = {v} must be in range [{o}, {o + (n - 1) * d}]")
        self._loc[axis] = v

    def _get(self, axis):
        if axis not in self._loc:
            raise RuntimeError(f"{axis} location not set")
        return self._loc[axis]

    def set_z_to_free_surface(self):
        self._set("z", self.geometry.z0)

    def clear(self):
        self._geometry = None
        self._loc = {}

    def __copy__(self):
        p = type(self)()
        p._geometry, p._loc = self._geometry, dict(self._loc)
        return p


class Source2D(_Point):
    x = property(lambda s: s._get("x"), lambda s, v: s._set("x", v))
    z = property(lambda s: s._get("z"), lambda s, v: s._set("z", v))


class Station2D(Source2D):
    pass


class Source3D(_Point):
    x = property(lambda s: s._get("x"), lambda s, v: s._set("x", v))
    y = property(lambda s: s._get("y"), lambda s, v: s._set("y", v))
    z = property(lambda s: s._get("z"), lambda s, v: s._set("z", v))


class Station3D(Source3D):
    pass


class _VelocityModel:
    _dim = 2

    def __init__(self):
        self._geometry = None
        self._v = None
        self._nodal = False
        self._ordering = 0

    def initialize(self, geometry):
        geometry._complete()
        self._geometry = geometry.__copy__()
        self._v = None

    @property
    def is_initialized(self):
        return self._geometry is not None

    @property
    def geometry(self):
        if self._geometry is None:
            raise RuntimeError("velocity model not initialized")
        return self._geometry

    def _sizes(self):
        g = self.geometry
        ns = (g.nx, g.nz) if self._dim == 2 else (g.nx, g.ny, g.nz)
        return int(np.prod(ns)), int(np.prod([n - 1 for n in ns]))

    def set_nodal_velocities(self, velocities, ordering=0):
        v = np.ascontiguousarray(velocities, dtype=np.float64).ravel()
        if v.size != self._sizes()[0]:
            raise ValueError(f"expecting {self._sizes()[0]} nodal velocities, got {v.size}")
        if not (v > 0).all():
            raise ValueError("Non-positive velocities detected")
        self._v, self._nodal, self._ordering = v, True, int(ordering)

    def set_cellular_velocities(self, velocities, ordering=0):
        v = np.ascontiguousarray(velocities, dtype=np.float64).ravel()
        if v.size != self._sizes()[1]:
            raise ValueError(f"expecting {self._sizes()[1]} cell velocities, got {v.size}")
        if not (v > 0).all():
            raise ValueError("Non-positive velocities detected")
        self._v, self._nodal, self._ordering = v, False, int(ordering)

    def __copy__(self):
        m = type(self)()
        m.__dict__.update(self.__dict__)
        return m

    def _upload(self, ctx):
        if self._v is None:
            raise RuntimeError("velocities not set")
        if self._dim == 2:
            (ctx.set_nodal_velocity2d(self._v, self._ordering) if self._nodal
             else ctx.set_slowness2d(1.0 / self._v, self._ordering))
        else:
            (ctx.set_nodal_velocity3d(self._v, self._ordering) if self._nodal
             else ctx.set_slowness3d(1.0 / self._v, self._ordering))

    def write_vtk(self, file_name, title="velocity_m/s"):
        g = self.geometry
        ny, dy, y0 = (1, 1.0, 0.0) if self._dim == 2 else (g.ny, g.dy, g.y0)
        with _vtk.RectilinearGridWriter(file_name, g.nx, ny, g.nz, g.dx, dy, g.dz, g.x0, y0, g.z0, title) as w:
            (w.nodal_scalars if self._nodal else w.cell_scalars)(title, self._v)


class VelocityModel2D(_VelocityModel):
    _dim = 2


class VelocityModel3D(_VelocityModel):
    _dim = 3


class _Solver:
    _dim = 2

    def __init__(self):
        self._ctx = None
        self._options = None
        self._geometry = None
        self._model = None
        self._source = None
        self._stations = []
        self._field = self._gradient = self._station_times = None

    def initialize(self, options, geometry):
        geometry._complete()
        self._options, self._geometry = options, geometry.__copy__()
        self._field = self._gradient = None

    def _context(self):
        if self._ctx is None:
            from . import Context
            self._ctx = Context(0)
        return self._ctx

    @property
    def velocity_model(self):
        if self._model is None:
            raise RuntimeError("velocity model not set")
        return self._model

    @velocity_model.setter
    def velocity_model(self, m):
        if self._geometry is None:
            raise RuntimeError("Class not initialized")
        if not m.is_initialized:
            raise ValueError("Velocity model not initialized")
        self._model = m.__copy__()
        self._field = self._gradient = None

    @property
    def source(self):
        if self._source is None:
            raise RuntimeError("Source location not set")
        return self._source

    @source.setter
    def source(self, s):
        if self._geometry is None:
            raise RuntimeError("Class not initialized")
        self._source = s.__copy__()
        self._field = self._gradient = None

    @property
    def stations(self):
        return list(self._stations)

    @stations.setter
    def stations(self, stations):
        self._stations = [s.__copy__() for s in stations]
        if self._field is not None:
            self._interpolate()

    have_source = property(lambda s: s._source is not None)
    have_velocity_model = property(lambda s: s._model is not None)
    have_travel_time_field = property(lambda s: s._field is not None)
    have_travel_time_gradient_field = property(lambda s: s._gradient is not None)

    @property
    def travel_time_field(self):
        if self._field is None:
            raise RuntimeError("Travel time field not yet computed")
        return self._field.copy()

    @property
    def travel_time_gradient_field(self):
        if self._gradient is None:
            raise RuntimeError("Travel time gradient field not computed")
        return self._gradient.copy()

    @property
    def travel_times_at_stations(self):
        if self._field is None:
            raise RuntimeError("Travel time field not yet computed")
        return list(self._station_times)


class Solver2D(_Solver):
    """The reference's Solver2D binding (python/pySolver2d.cpp:168-250), FP64."""

    def solve(self):
        from . import F64
        if self._geometry is None:
            raise RuntimeError("Class not initialized")
        g, m, s = self._geometry, self.velocity_model, self.source
        ctx = self._context()
        ctx.set_grid2d(g.nx, g.nz, g.dx, g.dz, g.x0, g.z0)
        m._upload(ctx)
        self._field = ctx.solve2d([(s.x, s.z)], self._options._options(), F64)[0].ravel()
        self._gradient = None
        self._interpolate()

    def _interpolate(self):
        self._station_times = (list(self._context().station_times2d([(q.x, q.z) for q in self._stations]))
                               if self._stations else [])

    def compute_travel_time_gradient_field(self):
        from . import F64
        if self._field is None:
            raise RuntimeError("Travel time field not yet computed")
        self._gradient = self._context().gradient2d(0, F64).ravel()

    def write_vtk(self, file_name, title="travel_time_field_s", write_gradient=False):
        g = self._geometry
        field = self.travel_time_field
        with _vtk.RectilinearGridWriter(file_name, g.nx, 1, g.nz, g.dx, 1.0, g.dz, g.x0, 0.0, g.z0, title) as w:
            w.nodal_scalars(title, field)
            if write_gradient:
                w.nodal_vectors(title + "_gradient", self.travel_time_gradient_field, 2)


class Solver3D(_Solver):
    """Solver2D's interface in 3D, FP64 (the reference's Solver3D, include/eikonalxx/solver3d.hpp)."""

    _dim = 3

    def solve(self):
        from . import F64
        if self._geometry is None:
            raise RuntimeError("Class not initialized")
        g, m, s = self._geometry, self.velocity_model, self.source
        ctx = self._context()
        ctx.set_grid3d(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, g.x0, g.y0, g.z0)
        m._upload(ctx)
        self._field = ctx.solve3d([(s.x, s.y, s.z)], self._options._options(), F64)[0].ravel()
        self._gradient = None
        self._interpolate()

    def _interpolate(self):
        self._station_times = (list(self._context().station_times3d([(q.x, q.y, q.z) for q in self._stations]))
                               if self._stations else [])

    def compute_travel_time_gradient_field(self):
        from . import F64
        if self._field is None:
            raise RuntimeError("Travel time field not yet computed")
        self._gradient = self._context().gradient3d(0, F64).ravel()

    def write_vtk(self, file_name, title="travel_time_field_s", write_gradient=False):
        g = self._geometry
        field = self.travel_time_field
        with _vtk.RectilinearGridWriter(file_name, g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, g.x0, g.y0, g.z0,
                                        title) as w:
            w.nodal_scalars(title, field)
            if write_gradient:
                w.nodal_vectors(title + "_gradient", self.travel_time_gradient_field, 3)


class Ray:
    """Ray-path value types of the reference's ray module (python/pyRay2d.cpp)."""

    class Point2D:
        def __init__(self):
            self.x = 0.0
            self.z = 0.0

        def clear(self):
            self.x = self.z = 0.0

        def __copy__(self):
            p = Ray.Point2D()
            p.x, p.z = self.x, self.z
            return p

    class Segment2D:
        def __init__(self):
            self.clear()

        def clear(self):
            self._start = self._end = None
            self._velocity = None
            self._cell = None

        def set_start_and_end_point(self, points):
            a, b = points
            self._start, self._end = a.__copy__(), b.__copy__()

        start_point = property(lambda s: s._start)
        end_point = property(lambda s: s._end)

        @property
        def length(self):
            return math.hypot(self._end.x - self._start.x, self._end.z - self._start.z)

        velocity = property(lambda s: s._velocity,
                            lambda s, v: setattr(s, "_velocity", _positive(v, "velocity")))
        velocity_model_cell_index = property(lambda s: s._cell,
                                             lambda s, v: setattr(s, "_cell", _at_least(v, 0, "cell index")))

        @property
        def travel_time(self):
            return self.length / self._velocity
