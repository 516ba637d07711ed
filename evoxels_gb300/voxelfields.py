"""``VoxelFields``: the host-side container of named 3-D fields and grid geometry.

Mirrors the reference's layout and geometry contract
(evoxels/voxelfields.py:28-194): NumPy fields of shape ``(Nx, Ny, Nz)``,
``spacing = domain_size / shape`` for cell-centred grids (``(Nx-1)`` cells in
x for ``staggered_x``), ``origin = spacing/2`` (``0`` in x for staggered),
default ``precision='float32'``.  Plotting is not provided (no graphics stack);
``export_to_vtk`` writes a legacy-ASCII VTK structured-points file.
"""

from __future__ import annotations

import warnings
from dataclasses import dataclass
from typing import Tuple

import numpy as np


@dataclass
class Grid:
    """Grid description handed to the backend (evoxels/voxelgrid.py:9-15)."""
    shape: Tuple[int, int, int]
    origin: Tuple[float, float, float]
    spacing: Tuple[float, float, float]
    convention: str


class VoxelFields:
    """Uniform voxel grid with named NumPy fields (evoxels/voxelfields.py:28-96)."""

    def __init__(self, shape, domain_size=(1, 1, 1), convention="cell_center"):
        if not (isinstance(shape, (list, tuple)) and len(shape) == 3
                and all(isinstance(n, (int, np.integer)) for n in shape)):
            raise ValueError("shape must be a tuple of three integers")
        self.shape = tuple(int(n) for n in shape)
        num_x, num_y, num_z = self.shape
        self.precision = "float32"
        self.convention = convention
        if not isinstance(domain_size, (list, tuple)) or len(domain_size) != 3:
            raise ValueError("domain_size must be a list or tuple with three elements (dx, dy, dz)")
        if not all(isinstance(x, (int, float)) for x in domain_size):
            raise ValueError("All elements in domain_size must be integers or floats")
        self.domain_size = domain_size
        if convention == "cell_center":
            self.spacing = (domain_size[0] / num_x, domain_size[1] / num_y, domain_size[2] / num_z)
            self.origin = (self.spacing[0] / 2, self.spacing[1] / 2, self.spacing[2] / 2)
        elif convention == "staggered_x":
            self.spacing = (domain_size[0] / (num_x - 1), domain_size[1] / num_y, domain_size[2] / num_z)
            self.origin = (0, self.spacing[1] / 2, self.spacing[2] / 2)
        else:
            raise ValueError("Chosen convention must be cell_center or staggered_x.")
        if np.max(self.spacing) / np.min(self.spacing) > 10:
            warnings.warn("Simulations become very questionable for largely different spacings e.g. dz >> dx.")
        self.grid = None
        self.fields = {}

    @property
    def Nx(self) -> int:
        return self.shape[0]

    @property
    def Ny(self) -> int:
        return self.shape[1]

    @property
    def Nz(self) -> int:
        return self.shape[2]

    def __str__(self):
        return (f"Domain with size {self.domain_size} and {self.shape} grid points on "
                f"{self.convention} position.")

    def grid_info(self) -> Grid:
        return Grid(self.shape, self.origin, self.spacing, self.convention)

    def set_field(self, name: str, array: np.ndarray):
        """Replace a field; shape must match (evoxels/voxelfields.py:123-143)."""
        if isinstance(array, np.ndarray):
            if array.shape == self.shape:
                self.fields[name] = array
            else:
                raise ValueError(f"The provided array must have the shape {self.shape}.")
        else:
            raise TypeError("The provided array must be a numpy array.")

    def add_field(self, name: str, array=None):
        if array is not None:
            self.set_field(name, array)
        else:
            self.set_field(name, np.zeros(self.shape))

    def set_voxel_sphere(self, name: str, center, radius, label=1):
        """Label voxels whose centres lie within ``radius`` (evoxels/voxelfields.py:158-169)."""
        x, y, z = np.ogrid[:self.Nx, :self.Ny, :self.Nz]
        d2 = (x * self.spacing[0] + self.origin[0] - center[0]) ** 2 + \
             (y * self.spacing[1] + self.origin[1] - center[1]) ** 2 + \
             (z * self.spacing[2] + self.origin[2] - center[2]) ** 2
        self.fields[name][d2 <= radius ** 2] = label

    def average(self, name: str):
        """Mean of a field; staggered grids count the end slabs as half cells."""
        if self.convention == "cell_center":
            return np.mean(self.fields[name])
        f = self.fields[name]
        avg = np.sum(f[1:-1, :, :]) + 0.5 * np.sum(f[0, :, :]) + 0.5 * np.sum(f[-1, :, :])
        return avg / ((self.Nx - 1) * self.Ny * self.Nz)

    def axes(self):
        return tuple(np.arange(0, n, dtype=self.precision) * self.spacing[i] + self.origin[i]
                     for i, n in enumerate(self.shape))

    def meshgrid(self):
        return tuple(np.meshgrid(*self.axes(), indexing="ij"))

    def export_to_vtk(self, filename="output.vtk", field_names=None, binary=True):
        """Write fields as cell data of a legacy VTK image (headless).

        Same geometry as the reference's pyvista ImageData
        (evoxels/voxelfields.py:196-214): ``(N+1)`` points per axis, origin at
        the lower cell corner, fields flattened in Fortran (x-fastest) order.
        ``binary`` (the default of pyvista's ``save``): big-endian float32
        payloads; ``binary=False`` writes ASCII.
        """
        if not str(filename).endswith(".vtk"):
            raise ValueError("filename must end with .vtk")
        names = field_names if field_names else list(self.fields.keys())
        nx, ny, nz = self.shape
        o = [self.origin[i] - self.spacing[i] / 2 for i in range(3)]
        head = ("# vtk DataFile Version 3.0\nevoxels_gb300 fields\n" + ("BINARY" if binary else "ASCII") +
                "\nDATASET STRUCTURED_POINTS\n" + f"DIMENSIONS {nx + 1} {ny + 1} {nz + 1}\n" +
                "ORIGIN {} {} {}\n".format(*o) + "SPACING {} {} {}\n".format(*self.spacing) +
                f"CELL_DATA {nx * ny * nz}\n")
        with open(filename, "wb") as f:
            f.write(head.encode())
            for name in names:
                data = np.asarray(self.fields[name], dtype=np.float32)
                f.write(f"SCALARS {name} float 1\nLOOKUP_TABLE default\n".encode())
                if binary:
                    f.write(np.ascontiguousarray(data.transpose(2, 1, 0), dtype=">f4").tobytes())
                    f.write(b"\n")
                else:
                    np.savetxt(f, data.flatten(order="F"), fmt="%.9g")

    def plot_slice(self, *args, **kwargs):
        raise NotImplementedError("plotting is not part of evoxels_gb300 (no graphics stack)")

    def plot_field_interactive(self, *args, **kwargs):
        raise NotImplementedError("plotting is not part of evoxels_gb300 (no graphics stack)")
