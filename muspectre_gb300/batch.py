"""Batched Newton-CG over many cells (RVEs or load cases).

``BatchSolver(cells, tol, maxiter, precision)`` solves every cell with the method of
``solvers.newton_cg``; the Newton steps of the cells run in lockstep and every CG
iteration is a single launch per spectral pass for all cells, replayed from one CUDA
graph.  Cells of one grid run the solo kernels with problem index = blockIdx.y, and
each cell's results are those of a solo ``newton_cg`` call on it, bit for bit.  Cells
of different grids (same dimension, formulation and material-law kind) run grouped
launches: each cell owns a range of the grid's blocks and its own FFT plans and
sizes (the generic pass kernels), with results equal to the solo ones within
rounding.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .solvers import OptimizeResult


class BatchSolver:
    def __init__(self, cells, tol, maxiter, precision='fp64', inner_tol=1e-2):
        if precision not in ('fp64', 'mixed'):
            raise ValueError("precision must be 'fp64' or 'mixed'")
        self.cells = list(cells)
        if not self.cells:
            raise ValueError('empty batch')
        for c in self.cells:
            c.initialise()
        arr = (C.c_void_p * len(self.cells))(*[c.handle.value for c in self.cells])
        h = C.c_void_p()
        L.check(L.lib().musg_batch_create(arr, len(self.cells), float(tol), int(maxiter),
                                          L.PRECISION_MIXED if precision == 'mixed' else L.PRECISION_FP64,
                                          C.byref(h)))
        self._h = h
        self.precision = precision
        if precision == 'mixed':
            L.check(L.lib().musg_batch_set_inner_tol(self._h, float(inner_tol)))

    def __del__(self):
        h = getattr(self, '_h', None)
        if h is not None and h.value:
            try:
                L.lib().musg_batch_destroy(h)
            except Exception:
                pass
            self._h = None

    def newton_cg(self, load_steps, newton_tol, equil_tol, return_stress=True):
        """load_steps: one D×D matrix for all cells, a list of matrices (the load path
        of every cell), or a list (per cell) of lists of matrices.  Returns, per cell,
        a list of OptimizeResult (one per step; ``grad`` is empty, use
        ``cell.get_strain()``)."""
        B = len(self.cells)
        d = self.cells[0].dim
        a = np.asarray(load_steps, dtype=np.float64)
        if a.ndim == 2:
            a = np.broadcast_to(a, (B, 1, d, d))
        elif a.ndim == 3:
            a = np.broadcast_to(a, (B,) + a.shape)
        if a.shape[0] != B or a.shape[-2:] != (d, d):
            raise ValueError('load steps must be (D, D), (steps, D, D) or (cells, steps, D, D)')
        ns = a.shape[1]
        flat = np.ascontiguousarray(a.transpose(0, 1, 3, 2)).reshape(-1)  # column-major matrices
        infos = (L.ResultInfo * (B * ns))()
        sizes = [c.nb_dof for c in self.cells]
        offs = np.concatenate([[0], np.cumsum([ns * n for n in sizes])]).astype(np.int64)
        flat_s = np.empty(int(offs[-1])) if return_stress else None  # cell after cell, ns x nb_dof each
        L.check(L.lib().musg_batch_newton_cg(self._h, L.dptr(flat), ns, float(newton_tol), float(equil_tol), infos,
                                             L.dptr(flat_s)))
        out = []
        for b in range(B):
            rs = []
            st_b = flat_s[offs[b]:offs[b + 1]].reshape(ns, sizes[b]) if return_stress else None
            for k in range(ns):
                i = infos[b * ns + k]
                rs.append(OptimizeResult(np.empty((0, 1)),
                                         st_b[k].reshape(-1, 1) if return_stress else np.empty((0, 1)),
                                         bool(i.success), int(i.status), i.message.decode(), int(i.nb_it),
                                         int(i.nb_fev), np.array(i.hom_stress[:d * d]).reshape(d, d).T))
            self.cells[b]._has_tangent = True
            out.append(rs)
        return out
