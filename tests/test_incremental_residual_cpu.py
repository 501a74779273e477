"""The design of the mixed path's incremental Newton residual, checked on the CPU with
the oracle's operators.  After the first (FP64) residual of a load step, the library
forms each later one as G(rhs - (P - P_k)) in FP32 (csrc/api.cpp, project_residual)
instead of accumulating rhs += G(-(P - P_k)) in FP64.  Here the FP32 projection is
emulated with scipy's single-precision FFTs around the oracle's Green operator (its
output rounded to FP32), on a small spheres cell over Newton steps with an inexact
inner solve (the oracle's SolverCG at 1e-2, as the mixed path's forcing term):

* projecting the previous residual minus the stress change keeps the part of the
  result outside the range of G at FP32 rounding of the result itself, which the fused
  FP32 CG iteration needs (it forms p.Ap as p.(K:p), true for p in that range);
* accumulating the projected changes leaves an out-of-range part that is rounding of
  the first change, so it grows relative to the shrinking residual;
* Newton with the projected scheme reaches the homogenised stress of FP64-projected
  residuals to 1e-7, with the same step count."""
import numpy as np
import pytest

from oracle import muspectre_oracle as o

sf = pytest.importorskip('scipy.fft')


def _proj32(cell, vec):
    pr = cell.projection
    d = pr.dim
    f = o.t2_from_vec(np.asarray(vec, dtype=np.float32), d).reshape(*pr.res, d, d).astype(np.float32)
    axes = tuple(range(d))
    fh = pr._apply_hat(sf.rfftn(f, axes=axes)).astype(np.complex64)
    out = sf.irfftn(fh, s=pr.res, axes=axes).astype(np.float32)
    return o.t2_to_vec(out.reshape(-1, d, d)).astype(np.float64)


def _run(scheme, n=16, steps=4):
    from muspectre_gb300 import workloads
    w = workloads.spheres(n)
    cell = o.Cell(w['res'], w['lengths'], o.FINITE_STRAIN, allow_even=True)
    for name, E, mask in (('inc', w['E_incl'], w['inside']), ('mat', w['E_matrix'], ~w['inside'])):
        m = cell.add_material(o.MaterialLinearElastic1(name, 3, E, w['nu']))
        m.pixels = list(np.flatnonzero(mask))
    cell.set_uniform_strain(np.eye(3) + w['load'])
    solver = o.SolverCG(cell, 1e-2, 4000)
    solver.initialise()
    Pk = rhs = None
    out_of_range, its = [], 0
    for it in range(steps):
        P, _ = cell.evaluate_stress_tangent()
        if scheme == 'fp64' or Pk is None:
            rhs = cell.apply_projection(-P)
        elif scheme == 'accumulate':
            rhs = rhs + _proj32(cell, -(P - Pk))
        else:
            rhs = _proj32(cell, rhs - (P - Pk))
        Pk = P.copy()
        out_of_range.append(np.linalg.norm(rhs - cell.apply_projection(rhs)) / np.linalg.norm(rhs))
        x = solver.solve(rhs)
        cell.F = cell.F + x
        its += 1
        if np.linalg.norm(x) / np.linalg.norm(cell.F) < 1e-6:
            break
    P, _ = cell.evaluate_stress_tangent()
    return o.homogenised(P, 3), out_of_range, its


def test_projected_difference_stays_in_range():
    ref, _, its64 = _run('fp64')
    hom, oor, its = _run('projected')
    assert max(oor) < 1e-6, oor
    assert its == its64
    assert np.linalg.norm(hom - ref) / np.linalg.norm(ref) < 1e-7


def test_accumulated_corrections_leave_the_range():
    _, oor, _ = _run('accumulate', steps=3)
    # 3e-6 after the first correction, 2e-4 after the second (the residual shrank ~100x)
    assert oor[2] > 30 * oor[1] > 0, oor
    assert oor[2] > 1e-4, oor
