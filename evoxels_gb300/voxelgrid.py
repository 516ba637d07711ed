"""CUDA backend grid: the role ``VoxelGridTorch`` plays in the reference.

``VoxelGridGB300`` holds the grid geometry and converts fields between NumPy
and CUDA tensors with the reference's layout (evoxels/voxelgrid.py:155-245):
``(C, Nx, Ny, Nz)`` float32, z fastest.  It also produces the C-ABI structs
(grid factors, boundary conditions) the kernels consume, computed with the
same float32 operations the reference uses (evoxels/voxelgrid.py:29-30).

Differences from the reference, on purpose: only CUDA devices and float32 are
accepted (there is no CPU fallback), and the grid does not call
``torch.set_default_device`` (no process-wide side effect).
"""

from __future__ import annotations

import warnings

import numpy as np
import torch

from . import _lib
from .voxelfields import Grid


def _require_cuda(device):
    dev = torch.device(device)
    if dev.type != "cuda":
        raise ValueError(f"evoxels_gb300 runs on CUDA devices only, got device={device!r}")
    if not torch.cuda.is_available():
        raise RuntimeError("evoxels_gb300 needs a CUDA GPU; torch.cuda.is_available() is False")
    if dev.index is None:
        dev = torch.device("cuda", torch.cuda.current_device())
    return dev


def grid_factors(spacing):
    """``div_dx``, ``div_dx2`` and ``sum(div_dx2)`` in float32 (evoxels/voxelgrid.py:29-30)."""
    sp = torch.tensor(np.array(spacing, dtype=np.float64), dtype=torch.float32)
    div_dx = 1 / sp
    div_dx2 = 1 / sp ** 2
    return div_dx, div_dx2, torch.sum(div_dx2)


class CellCenteredBCs:
    """Ghost padding utilities (evoxels/boundary_conditions.py:5-82).

    The stencil kernels apply ghosts in-kernel; these tensor versions exist
    for API parity (frame export, user code) and are not on the hot path.
    """

    def __init__(self, vg):
        self.vg = vg

    def pad_periodic(self, field):
        return self.vg.pad_periodic(field)

    def pad_dirichlet_periodic(self, field, bc0=0, bc1=0):
        padded = self.vg.pad_periodic(field)
        padded[:, 0] = 2.0 * bc0 - padded[:, 1]
        padded[:, -1] = 2.0 * bc1 - padded[:, -2]
        return padded

    def pad_zero_flux_periodic(self, field):
        padded = self.vg.pad_periodic(field)
        padded[:, 0] = padded[:, 1]
        padded[:, -1] = padded[:, -2]
        return padded

    def pad_bc(self, field, bc):
        padded = self.vg.pad_periodic(field)
        for axis, (kind, values) in enumerate(bc):
            if kind == "periodic":
                continue
            lo = [slice(None)] * 4
            hi = [slice(None)] * 4
            lo_in = [slice(None)] * 4
            hi_in = [slice(None)] * 4
            lo[axis + 1], hi[axis + 1], lo_in[axis + 1], hi_in[axis + 1] = 0, -1, 1, -2
            if kind == "neumann":
                padded[tuple(lo)] = padded[tuple(lo_in)]
                padded[tuple(hi)] = padded[tuple(hi_in)]
            elif kind == "dirichlet":
                padded[tuple(lo)] = 2.0 * values[0] - padded[tuple(lo_in)]
                padded[tuple(hi)] = 2.0 * values[1] - padded[tuple(hi_in)]
            else:
                raise ValueError(f"Unsupported BC type: {kind}")
        return padded

    def pad_fft_periodic(self, field):
        return field

    def pad_fft_dirichlet_periodic(self, field):
        """Pad with the negated x-flipped field (evoxels/boundary_conditions.py:64-66)."""
        return torch.cat((field, -torch.flip(field, [1])), 1)

    def pad_fft_zero_flux_periodic(self, field):
        """Pad with the x-flipped field (evoxels/boundary_conditions.py:68-70)."""
        return torch.cat((field, torch.flip(field, [1])), 1)

    def trim_boundary_nodes(self, field):
        return field

    def trim_ghost_nodes(self, field):
        if field[0, 1:-1, 1:-1, 1:-1].shape == self.vg.shape:
            return field[:, 1:-1, 1:-1, 1:-1]
        raise ValueError(f"The provided field has the wrong shape {self.vg.shape}.")


class VoxelGridGB300:
    """Grid geometry + CUDA field conversion (evoxels/voxelgrid.py:18-245)."""

    def __init__(self, grid: Grid, precision="float32", device="cuda"):
        if precision != "float32":
            raise NotImplementedError("evoxels_gb300 kernels compute in float32 only")
        if grid.convention != "cell_center":
            raise NotImplementedError("evoxels_gb300 implements the cell_center convention only")
        self.shape = tuple(int(n) for n in grid.shape)
        self.origin = grid.origin
        self.spacing = tuple(float(h) for h in grid.spacing)
        self.convention = grid.convention
        self.device = _require_cuda(device)
        self.precision = torch.float32
        self.lib = torch
        dx, dx2, s2 = grid_factors(self.spacing)
        self._factors = (dx, dx2, s2)
        self.div_dx = dx.to(self.device)
        self.div_dx2 = dx2.to(self.device)
        self.bc = CellCenteredBCs(self)

    # ---- conversion (evoxels/voxelgrid.py:126-135,188-192) --------------------
    def to_backend(self, np_arr):
        return torch.tensor(np_arr, dtype=self.precision, device=self.device)

    def to_numpy(self, field):
        return field.detach().cpu().numpy()

    def init_scalar_field(self, array):
        return self.to_backend(array).unsqueeze(0)

    def export_scalar_field_to_numpy(self, field):
        return self.to_numpy(torch.squeeze(field, 0))

    def concatenate(self, fieldlist, dim):
        return torch.cat(fieldlist, dim=dim)

    def pad_periodic(self, field):
        return torch.nn.functional.pad(field, (1, 1, 1, 1, 1, 1), mode="circular")

    def pad_zeros(self, field):
        return torch.nn.functional.pad(field, (1, 1, 1, 1, 1, 1), mode="constant", value=0)

    def set(self, field, index, value):
        field[index] = value
        return field

    # ---- spectral grids (evoxels/voxelgrid.py:84-114) ----------------------------
    def fft_axes(self):
        return tuple(2 * torch.pi * torch.fft.fftfreq(n, h, dtype=torch.float32, device=self.device)
                     for n, h in zip(self.shape, self.spacing))

    def rfft_axes(self):
        return tuple(2 * torch.pi * torch.fft.rfftfreq(n, h, dtype=torch.float32, device=self.device)
                     for n, h in zip(self.shape, self.spacing))

    def rfft_k_squared(self):
        a_x, a_y, _ = self.fft_axes()
        _, _, a_z = self.rfft_axes()
        kx, ky, kz = torch.meshgrid(a_x, a_y, a_z, indexing="ij")
        return kx ** 2 + ky ** 2 + kz ** 2

    def rfft_k_squared_nonperiodic(self):
        """k^2 of the x-mirrored grid, 2*Nx points along x (evoxels/voxelgrid.py:116-124)."""
        a_x = 2 * torch.pi * torch.fft.fftfreq(2 * self.shape[0], d=self.spacing[0], device=self.device)
        _, a_y, _ = self.fft_axes()
        _, _, a_z = self.rfft_axes()
        kx, ky, kz = torch.meshgrid(a_x, a_y, a_z, indexing="ij")
        return kx ** 2 + ky ** 2 + kz ** 2

    # ---- C-ABI structs ------------------------------------------------------------
    def evx_grid(self):
        dx, dx2, s2 = self._factors
        g = _lib.EvxGrid()
        g.nx, g.ny, g.nz = self.shape
        for a in range(3):
            g.h[a] = self.spacing[a]
            g.inv_h[a] = float(dx[a])
            g.inv_h2[a] = float(dx2[a])
        g.inv_h2_sum = float(s2)
        return g

    def check_field(self, u):
        """Validate a state tensor against this grid (evoxels/boundary_conditions.py:76-82)."""
        if not isinstance(u, torch.Tensor):
            raise TypeError("fields must be torch tensors on the grid's CUDA device")
        if u.dim() != 4 or tuple(u.shape[1:]) != self.shape:
            raise ValueError(f"The provided field has the wrong shape {tuple(u.shape)}; expected "
                             f"(C, {self.shape[0]}, {self.shape[1]}, {self.shape[2]}).")
        if u.dtype != torch.float32:
            raise TypeError(f"fields must be float32, got {u.dtype}")
        if u.device != self.device:
            raise ValueError(f"field is on {u.device}, grid is on {self.device}")
        return u.contiguous()


def evx_bc(bc):
    """Normalised reference BC tuple -> ``EvxBC`` (Dirichlet ghost = float32(2*v) - cell)."""
    s = _lib.EvxBC()
    for a, (kind, values) in enumerate(bc):
        s.kind[a] = _lib.BC_CODES[kind]
        if kind == "dirichlet":
            s.two_v_lo[a] = float(np.float32(2.0 * values[0]))
            s.two_v_hi[a] = float(np.float32(2.0 * values[1]))
    return s


def cuda_stream():
    return torch.cuda.current_stream().cuda_stream


def normalize_bc(bc, convention="cell_center"):
    """BC normalisation and validation (evoxels/problem_definition.py:60-103)."""
    if bc is None or bc == "fully_periodic":
        return (("periodic", None),) * 3
    if len(bc) != 3:
        raise ValueError("bc must contain exactly three axis entries ordered as (x, y, z).")
    out = []
    for axis_bc in bc:
        if isinstance(axis_bc, str):
            if axis_bc == "dirichlet":
                raise ValueError("Dirichlet BCs require explicit values ('dirichlet', (left, right)).")
            if axis_bc not in {"periodic", "neumann"}:
                raise ValueError(f"Unsupported BC type: {axis_bc}")
            out.append((axis_bc, None))
            continue
        if len(axis_bc) != 2:
            raise ValueError("Each axis boundary specification must be either a string or "
                             "a tuple like ('dirichlet', (left, right)).")
        kind, values = axis_bc
        if kind not in {"periodic", "dirichlet", "neumann"}:
            raise ValueError(f"Unsupported BC type: {kind}")
        if kind == "dirichlet":
            if values is None or len(values) != 2:
                raise ValueError("Dirichlet BCs require two boundary values.")
            if convention == "cell_center":
                warnings.warn("Applying Dirichlet BCs on a cell_center grid "
                              "reduces the spatial order of convergence to 0.5!")
            out.append((kind, tuple(values)))
        else:
            if values is not None:
                raise ValueError(f"{kind} BCs do not accept boundary values.")
            out.append((kind, None))
    return tuple(out)
