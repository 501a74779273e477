"""Solvers (language_bindings/python/bind_py_solvers.cc:52-156).

``SolverCG(cell, tol, maxiter, verbose=False)`` keeps its vectors on the GPU;
``precision='mixed'`` runs the CG, FFTs, projection and tangent in FP32 with
compensated dot products while the Newton level (residual, increments, stress,
return mapping) stays FP64.  The FP32 inner solve stops at max(tol, inner_tol)
(default 1e-2, the forcing term of an inexact Newton method: each Newton step
contracts the error by about inner_tol and the FP64 Newton loop refines to
newton_tol, which takes fewer CG iterations in total than tight inner solves) and
the FP64 Newton loop refines; for history-free materials the returned stress is
evaluated at the returned strain.  The Newton residual G(-P) is projected in FP64
once per load step; later ones are the FP32 projection of the previous residual
minus the stress change since (``incremental_residual=False`` projects every
residual in FP64).  ``newton_cg`` follows
src/solver/solvers.cc:44-217.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import _lib as L
from ._lib import ConvergenceError, SolverError  # noqa: F401


@dataclass
class OptimizeResult:
    """src/solver/solver_common.hh:50-67 (grad and stress are (nb_dof, 1) arrays), plus
    ``hom_stress``: the pixel mean of the stress after the load step (D×D, reduced on
    the device; available with ``return_fields=False`` too)."""
    grad: np.ndarray
    stress: np.ndarray
    success: bool
    status: int
    message: str
    nb_it: int
    nb_fev: int
    hom_stress: Optional[np.ndarray] = None


class SolverBase:
    pass


class SolverCG(SolverBase):
    """SolverCG (src/solver/solver_cg.hh:51-106, solver_cg.cc:54-110)."""

    def __init__(self, cell, tol, maxiter, verbose=False, precision='fp64', inner_tol=1e-2,
                 incremental_residual=True):
        if precision not in ('fp64', 'mixed'):
            raise ValueError("precision must be 'fp64' or 'mixed'")
        self.cell = cell
        self.tol = float(tol)
        self.maxiter = int(maxiter)
        self.verbose = bool(verbose)
        self.precision = precision
        h = C.c_void_p()
        L.check(L.lib().musg_solver_cg_create(cell.handle, self.tol, self.maxiter, int(self.verbose),
                                              L.PRECISION_MIXED if precision == 'mixed' else L.PRECISION_FP64,
                                              C.byref(h)))
        self._h = h
        self.inner_tol = float(inner_tol)
        self.incremental_residual = bool(incremental_residual)
        if precision == 'mixed':
            L.check(L.lib().musg_solver_set_inner_tol(self._h, self.inner_tol))
            L.check(L.lib().musg_solver_set_incremental_residual(self._h, int(self.incremental_residual)))

    def __del__(self):
        h = getattr(self, '_h', None)
        if h is not None and h.value:
            try:
                L.lib().musg_solver_destroy(h)
            except Exception:
                pass
            self._h = None

    @property
    def handle(self):
        return self._h

    def name(self):
        return 'CG'

    def get_name(self):
        return 'CG'

    def get_tol(self):
        return self.tol

    def get_maxiter(self):
        return self.maxiter

    def get_counter(self):
        c = C.c_uint(0)
        L.check(L.lib().musg_solver_get_counter(self._h, C.byref(c)))
        return c.value

    def reset_counter(self):
        L.check(L.lib().musg_solver_reset_counter(self._h))

    def has_converged(self):
        c = C.c_int(0)
        L.check(L.lib().musg_solver_has_converged(self._h, C.byref(c)))
        return bool(c.value)

    def initialise(self):
        pass

    def profile(self, iterations=5):
        """Mean per-kernel duration (ms) of one CG iteration, CUDA events on the
        cell's stream, from the cell's last residual: {kernel name: ms}."""
        ms = np.zeros(16)
        nk = C.c_int(0)
        L.check(L.lib().musg_solver_profile(self._h, int(iterations), L.dptr(ms), C.byref(nk)))
        return {L.lib().musg_solver_kernel_name(self._h, k).decode(): float(ms[k]) for k in range(nk.value)}

    def solve(self, rhs):
        """SolverCG::solve on a flat host vector; returns x."""
        b = L.f64(np.asarray(rhs).reshape(-1))
        x = np.empty_like(b)
        L.check(L.lib().musg_solver_solve(self._h, L.dptr(b), L.dptr(x)))
        return x


def newton_cg(cell, load_steps, solver, newton_tol, equil_tol=None, verbose=0, *, return_fields=True,
              line_search=False, **kw):
    """newton_cg(cell, ΔF₀ | [ΔF...], solver, newton_tol, equil_tol, verbose=0)
    (bind_py_solvers.cc:75-106).  A single D×D load returns one OptimizeResult, a
    list returns a list.  ``return_fields=False`` skips the per-step copies of the
    strain and stress fields to the host (the arrays are then empty).

    ``line_search=True`` (an extension, off by default) damps every Newton increment
    by a backtracking line search on the norm of the projected residual: F = F0 + λ δF
    with λ = 1, 1/2, ... until the norm falls below (1 - 1e-4 λ) of the current one
    (or λ = 1/1024).  The convergence test still measures the full increment δF, and
    a load step takes at most min(maxiter, 100) Newton iterations.  It is what makes
    the consistent elasto-plastic tangent converge on heterogeneous cells under large
    load increments."""
    L.check(L.lib().musg_solver_set_line_search(solver.handle, 1 if line_search else 0))
    return _newton('musg_newton_cg', cell, load_steps, solver, newton_tol, equil_tol, verbose, return_fields, kw)


def de_geus(cell, load_steps, solver, newton_tol, equil_tol=None, verbose=0, *, return_fields=True,
            line_search=False, **kw):
    """de_geus(cell, ΔF₀ | [ΔF...], solver, newton_tol, equil_tol, verbose=0)
    (bind_py_solvers.cc:108-138, solvers.cc:220-408): each load step starts with the
    response to the macroscopic increment at the previous equilibrium.
    ``line_search=True`` (an extension, off by default) damps the later Newton
    increments of a load step as in :func:`newton_cg`."""
    L.check(L.lib().musg_solver_set_line_search(solver.handle, 1 if line_search else 0))
    return _newton('musg_de_geus', cell, load_steps, solver, newton_tol, equil_tol, verbose, return_fields, kw)


def _newton(entry, cell, load_steps, solver, newton_tol, equil_tol, verbose, return_fields, kw):
    if equil_tol is None:
        equil_tol = kw.pop('equilibrium_tol')
    single = not isinstance(load_steps, (list, tuple))
    steps = [np.asarray(load_steps, dtype=np.float64)] if single else [np.asarray(s, dtype=np.float64)
                                                                     for s in load_steps]
    d = cell.dim
    for s in steps:
        if s.shape != (d, d):
            raise SolverError('Load increments need to be given in {0}×{0} matrices, but I got a {1} matrix'.format(
                d, '×'.join(str(x) for x in s.shape)))
    cell.initialise()
    n = len(steps)
    flat = L.f64(np.stack([s.T.reshape(-1) for s in steps]))  # column-major matrices
    infos = (L.ResultInfo * n)()
    grads = np.empty((n, cell.nb_dof)) if return_fields else None
    stresses = np.empty((n, cell.nb_dof)) if return_fields else None
    L.check(getattr(L.lib(), entry)(cell.handle, L.dptr(flat), n, solver.handle, float(newton_tol), float(equil_tol),
                                    int(verbose), infos, L.dptr(grads), L.dptr(stresses)))
    cell._has_tangent = True
    out = []
    for k in range(n):
        i = infos[k]
        out.append(OptimizeResult(grads[k].reshape(-1, 1) if return_fields else np.empty((0, 1)),
                                  stresses[k].reshape(-1, 1) if return_fields else np.empty((0, 1)),
                                  bool(i.success), int(i.status), i.message.decode(), int(i.nb_it), int(i.nb_fev),
                                  np.array(i.hom_stress[:d * d]).reshape(d, d).T))
    return out[0] if single else out
