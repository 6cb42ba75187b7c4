"""Legacy-VTK rectilinear-grid files of travel-time fields, velocity models and gradients.

The file layout is that of the reference's writer (src/io/vtkRectilinearGrid2d.cpp,
src/io/vtkRectilinearGrid3d.cpp, src/io/pack.hpp), so files open the same way in
ParaView / VisIt: the "# vtk DataFile Version 3.0" header, the title with blanks replaced
by underscores, BINARY (big-endian float32) or ASCII, DATASET RECTILINEAR_GRID with
X/Y/Z_COORDINATES (z written as -depth, as the reference does for its binary files),
then POINT_DATA (nodal scalars, "LOOKUP_TABLE default" once, nodal vectors) and
CELL_DATA (cellular scalars).  A 2D grid is written with one y coordinate.
"""
import os

import numpy as np


def _name(s, default):
    s = s if s else default
    return "".join("_" if c.isspace() else c for c in s)


class RectilinearGridWriter:
    """Writes one rectilinear grid file; datasets are appended in call order."""

    def __init__(self, path, nx, ny, nz, dx, dy, dz, x0=0.0, y0=0.0, z0=0.0, title="", binary=True):
        parent = os.path.dirname(os.path.abspath(path))
        os.makedirs(parent, exist_ok=True)
        self.n = (int(nx), int(ny), int(nz))
        self.binary = binary
        self._wrote_points = self._wrote_cells = self._wrote_lut = False
        self.f = open(path, "wb")
        xs = x0 + dx * np.arange(nx)
        ys = y0 + dy * np.arange(ny) if ny > 1 else np.zeros(1)
        zs = -(z0 + dz * np.arange(nz))
        self._line("# vtk DataFile Version 3.0")
        self._line(_name(title, "vtk_dataset"))
        self._line("BINARY" if binary else "ASCII")
        self._line("DATASET RECTILINEAR_GRID")
        self._line(f"DIMENSIONS {nx} {ny} {nz}")
        for axis, c in (("X", xs), ("Y", ys), ("Z", zs)):
            self._line(f"{axis}_COORDINATES {len(c)} float")
            self._values(c)

    def _line(self, s):
        self.f.write((s + "\n").encode())

    def _values(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64).ravel()
        if self.binary:
            self.f.write(a.astype(">f4").tobytes())
            self.f.write(b"\n")
        else:
            for v in a.astype(np.float32):
                self._line(repr(float(v)))

    def nodal_scalars(self, name, values):
        """values: natural order (z slowest, x fastest), nx*ny*nz entries."""
        if not self._wrote_points:
            self._line(f"POINT_DATA {np.prod(self.n)}")
            self._wrote_points = True
        self._line(f"SCALARS {_name(name, 'dataset')} float 1")
        if not self._wrote_lut:
            self._line("LOOKUP_TABLE default")
            self._wrote_lut = True
        self._values(values)

    def nodal_vectors(self, name, values, components):
        """values: interleaved per node with `components` entries (2: (x, z), 3: (x, y, z))."""
        if not self._wrote_points:
            self._line(f"POINT_DATA {np.prod(self.n)}")
            self._wrote_points = True
        v = np.asarray(values, dtype=np.float64).reshape(-1, components)
        if components == 2:
            v = np.column_stack([v[:, 0], np.zeros(len(v)), v[:, 1]])
        self._line(f"VECTORS {_name(name, 'vector_dataset')} float")
        self._values(v)

    def cell_scalars(self, name, values):
        nc = int(np.prod([max(1, k - 1) for k in self.n]))
        if not self._wrote_cells:
            self._line(f"CELL_DATA {nc}")
            self._wrote_cells = True
        self._line(f"SCALARS {_name(name, 'dataset')} float 1")
        self._line("LOOKUP_TABLE default")
        self._values(values)

    def close(self):
        if self.f:
            self.f.close()
            self.f = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

