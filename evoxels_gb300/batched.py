"""Batched uneven Cahn-Hilliard instances on one GPU.

Many independent periodic grids of different shapes, each with its own
mobility ``D`` and gradient parameter ``eps`` (``kappa = 2*eps``), advance
together: one persistent stencil launch over all instances' tiles, cuFFT
batched per shape group, one k-space launch, with runs of steps replayed from
a captured CUDA graph (``evx_batch_*`` in ``include/evx.h``).  The reference
batches same-shape solves with ``jax.vmap`` for parameter estimation
(evoxels/inversion.py:105-124); here the shapes may differ.

Fields are exchanged as one packed float32 CUDA tensor; ``pack``/``unpack``
convert from / to per-instance ``(1, Nx, Ny, Nz)`` tensors.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from .partition import shard
from .problem_definition import ch_params, double_well_coefficient
from .voxelgrid import _require_cuda, cuda_stream, grid_factors


@dataclass
class BatchTuning:
    """Knobs of the batched path (chosen by ``autotune.tune_batched``)."""
    tile_variant: int = -1    # -1 automatic per instance, 0 = 16x64, 1 = 32x32
    x_chunk: int = 0          # x planes per work item (0 = automatic)
    blocks_per_sm: int = 0    # persistent blocks per SM (0 = occupancy limit)
    fft_group_max: int = 0    # instances per cuFFT plan (0 = whole shape group)
    graph_steps: int = 20     # fused steps per captured CUDA graph (0 = no graph)

    def to_c(self):
        t = _lib.EvxBatchTuning()
        t.tile_variant, t.x_chunk, t.blocks_per_sm = self.tile_variant, self.x_chunk, self.blocks_per_sm
        t.fft_group_max, t.graph_steps = self.fft_group_max, self.graph_steps
        return t


class BatchedCahnHilliard:
    """``n`` periodic Cahn-Hilliard instances stepped with the IMEX scheme.

    ``shapes``: list of ``(Nx, Ny, Nz)`` (Nz % 4 == 0); ``D``, ``eps``: per
    instance (scalars broadcast); ``mu_hom``: ``None`` (bulk ``18/eps``) or a
    double-well callable pinning the bulk coefficient for every instance;
    ``spacing``: per-instance spacing (default 1).
    """

    def __init__(self, shapes, D=1.0, eps=3.0, dt=0.1, A=0.25, mu_hom=None, spacing=None,
                 tuning: BatchTuning | None = None, device="cuda", cufft3d=False, cufft_yz=False, z_pass=False):
        self.device = _require_cuda(device)
        self.shapes = [tuple(int(x) for x in s) for s in shapes]
        n = len(self.shapes)
        self.n = n
        self.D = np.broadcast_to(np.asarray(D, dtype=np.float64), (n,)).copy()
        self.eps = np.broadcast_to(np.asarray(eps, dtype=np.float64), (n,)).copy()
        self.dt, self.A = float(dt), float(A)
        self.pinned_w = None if mu_hom is None else double_well_coefficient(mu_hom, 1.0)
        self.spacing = [tuple(map(float, s)) for s in (spacing or [(1.0, 1.0, 1.0)] * n)]
        self.tuning = tuning or BatchTuning()
        inst = (_lib.EvxBatchInstance * n)()
        for i, (shape, h) in enumerate(zip(self.shapes, self.spacing)):
            dx, dx2, s2 = grid_factors(h)
            inst[i].nx, inst[i].ny, inst[i].nz = shape
            for a in range(3):
                inst[i].h[a] = h[a]
                inst[i].inv_h[a] = float(dx[a])
                inst[i].inv_h2[a] = float(dx2[a])
            inst[i].inv_h2_sum = float(s2)
            inst[i].params = ch_params(self.eps[i], self.D[i], self.A, self.dt, self.pinned_w)
        self._inst = inst
        h = C.c_void_p()
        L = _lib.lib()
        with torch.cuda.device(self.device):
            # flags bit 1: cuFFT 3-D for every shape group (default: power-of-two nx groups
            # use cuFFT (y, z) plus the batched x-pass)
            flags = (2 if cufft3d else 0) | (8 if cufft_yz else 0) | (16 if z_pass else 0)
            _lib.check(L.evx_batch_create(C.byref(h), inst, n, self.tuning.to_c(), flags),
                       "evx_batch_create")
        self.handle = h
        self.total = int(L.evx_batch_field_floats(h))
        self.work_items = int(L.evx_batch_work_items(h))
        offs = (C.c_int64 * n)()
        _lib.check(L.evx_batch_offsets(h, offs), "evx_batch_offsets")
        self.offsets = [int(o) for o in offs]
        self.sizes = [int(np.prod(s)) for s in self.shapes]
        self.workspace = torch.empty(int(L.evx_batch_workspace_bytes(h)), dtype=torch.uint8, device=self.device)

    @classmethod
    def for_rank(cls, shapes, rank, world_size, D=1.0, eps=3.0, **kw):
        """The instances this rank advances when a batch is sharded over ``world_size`` GPUs, one
        process per GPU: ``partition_instances(shapes, world_size)[rank]`` (balanced by voxel count,
        the same split on every rank; independent instances need no collective).  ``D`` and ``eps``
        are for the whole batch; ``global_index`` maps the shard's instances to positions in
        ``shapes``, and ``pack_shard(fields)`` packs this rank's fields from the whole list."""
        idx, sub, d, e = shard(shapes, rank, world_size, D, eps)
        b = cls(sub, d, e, **kw)
        b.global_index = idx
        return b

    def pack_shard(self, fields, out=None):
        """Pack this shard's instances from the fields of the whole batch (see ``for_rank``)."""
        return self.pack([fields[i] for i in getattr(self, "global_index", range(len(fields)))], out)

    def __del__(self):
        try:
            if getattr(self, "handle", None):
                _lib.lib().evx_batch_destroy(self.handle)
                self.handle = None
        except Exception:  # noqa: BLE001 - interpreter shutdown
            pass

    @property
    def voxels(self):
        return sum(self.sizes)

    # ---- packing ---------------------------------------------------------------
    def empty(self):
        return torch.zeros(self.total, dtype=torch.float32, device=self.device)

    def pack(self, fields, out=None):
        """Per-instance fields (NumPy or tensors, shape (Nx,Ny,Nz) or (1,Nx,Ny,Nz)) -> packed tensor."""
        out = self.empty() if out is None else out
        for f, o, n, s in zip(fields, self.offsets, self.sizes, self.shapes):
            t = torch.as_tensor(f, dtype=torch.float32).reshape(s)
            out[o:o + n].view(s).copy_(t)
        return out

    def unpack(self, packed):
        """Packed tensor -> list of ``(1, Nx, Ny, Nz)`` views."""
        return [packed[o:o + n].view((1,) + s) for o, n, s in zip(self.offsets, self.sizes, self.shapes)]

    # ---- stepping --------------------------------------------------------------
    def new_spectra(self, nsteps):
        """Buffer for ``nsteps`` steps of stored increment spectra (every instance)."""
        n = int(_lib.lib().evx_batch_spectrum_floats(self.handle))
        return torch.empty(max(1, int(nsteps) * n), dtype=torch.float32, device=self.device)

    def _check_spectra(self, spectra, nsteps):
        n = int(_lib.lib().evx_batch_spectrum_floats(self.handle))
        if spectra.dtype != torch.float32 or not spectra.is_contiguous() or spectra.numel() < int(nsteps) * n:
            raise ValueError("spectra must be a contiguous float32 tensor from new_spectra(nsteps)")

    def forward(self, u, nsteps, traj=None, nonfinite=None, spectra=None):
        """``nsteps`` IMEX steps of every instance; ``traj`` (nsteps x total) receives u_1..u_n,
        ``spectra`` (optional, from ``new_spectra``; needs ``traj``) each step's increment spectra."""
        self._check(u)
        out = torch.empty_like(u)
        if traj is not None:
            self._check(traj, nsteps)
        if spectra is not None:
            self._check_spectra(spectra, nsteps)
        _lib.check(_lib.lib().evx_batch_forward_spectra(self.handle, u.data_ptr(), out.data_ptr(), int(nsteps),
                                                        traj.data_ptr() if traj is not None else None,
                                                        spectra.data_ptr() if spectra is not None else None,
                                                        nonfinite.data_ptr() if nonfinite is not None else None,
                                                        self.workspace.data_ptr(), cuda_stream()),
                   "evx_batch_forward_spectra")
        return out

    def adjoint(self, states, nsteps, lam, grads=None, spectra=None):
        """Adjoint through ``states`` ((nsteps+1) x total); ``grads`` (n x 3 float64) accumulates.
        ``spectra``: the forward's stored spectra of the same steps (the mobility gradient sums then
        come from k-space by Parseval)."""
        self._check(states, nsteps + 1)
        self._check(lam)
        if spectra is not None:
            self._check_spectra(spectra, nsteps)
        out = torch.empty_like(lam)
        _lib.check(_lib.lib().evx_batch_adjoint_spectra(self.handle, states.data_ptr(),
                                                        spectra.data_ptr() if spectra is not None else None,
                                                        int(nsteps), lam.data_ptr(), out.data_ptr(),
                                                        grads.data_ptr() if grads is not None else None,
                                                        self.workspace.data_ptr(), cuda_stream()),
                   "evx_batch_adjoint_spectra")
        return out

    def param_grads(self, grads):
        """(dL/dD, dL/dkappa, dL/dw) per instance -> (dL/dD, dL/deps)."""
        g = grads.detach().cpu().numpy()
        _lib.check_device_status("BatchedCahnHilliard gradients")
        geps = 2.0 * g[:, 1]
        if self.pinned_w is None:
            geps = geps - 18.0 / self.eps ** 2 * g[:, 2]
        return g[:, 0].copy(), geps

    def _check(self, t, rows=1):
        if t.dtype != torch.float32 or not t.is_contiguous() or t.device != self.device:
            raise ValueError("batched buffers must be contiguous float32 tensors on the batch's device")
        if t.numel() < rows * self.total:
            raise ValueError(f"buffer holds {t.numel()} floats, needs {rows * self.total}")
