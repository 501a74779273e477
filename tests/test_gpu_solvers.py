"""de_geus (solvers.cc:220-408) on the GPU against the oracle's restatement.

Criteria follow test_gpu_parity.py: the README case (2-D) with identical Newton and
CG counts and fields within 1e-10; an odd 3-D grid over two load steps (the second
step starts from the first one's equilibrium) with identical Newton counts, CG counts
within 1%, the strain field within 1e-10 and the stress within the oracle's own
FFT-rounding spread; the reference's laminate patch test with exact layer strains;
the mixed-precision solve within 1e-6 of FP64 in homogenised stress.
"""
import numpy as np
import pytest

from oracle import muspectre_oracle as o

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def mu():
    import muspectre_gb300 as m
    if m.device_count() < 1:
        pytest.fail('no CUDA device visible')
    return m


def rel(a, b):
    a, b = np.asarray(a).reshape(-1), np.asarray(b).reshape(-1)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_laminate_patch_de_geus_gpu(mu):
    """test_solver_newton_cg.cc:218-323: exact layer strains to 1e-12."""
    res = [3, 3]
    cell = mu.Cell(res, [1., 1.], mu.Formulation.small_strain)
    hard = mu.material.MaterialLinearElastic1_2d.make(cell, 'hard', 4.0, .33)
    soft = mu.material.MaterialLinearElastic1_2d.make(cell, 'soft', 2.0, .33)
    for pixel in cell:
        (hard if pixel[0] < 1 else soft).add_pixel(pixel)
    factor = 1 / 2 * 1 / 3 + 1. - 1 / 3.
    eps_soft = 1.0 / factor
    eps_hard = eps_soft / 2
    for pattern in (np.array([[1., 0], [0, 0]]), np.array([[0, 1.], [1., 0]])):
        r = mu.solvers.de_geus(cell, pattern, mu.solvers.SolverCG(cell, 1e-8, 20), 1e-5, 1e-10)
        assert r.success
        F = r.grad.reshape(-1, 2, 2).transpose(0, 2, 1)
        for i, pixel in enumerate(cell):
            ref = (eps_hard if pixel[0] < 1 else eps_soft) * pattern
            assert np.linalg.norm(F[i] - ref) <= 1e-12


def test_readme_case_de_geus(mu):
    import test_gpu_parity as tp
    ocell, gcell = tp._readme_pair(mu)
    Del0 = np.array([[.0, .0], [0, .03]])
    ro = o.de_geus(ocell, Del0, o.SolverCG(ocell, 1e-8, 401), 1e-5, 2, 0)
    rg = mu.solvers.de_geus(gcell, Del0, mu.solvers.SolverCG(gcell, 1e-8, 401), 1e-5, 2)
    assert (rg.nb_it, rg.nb_fev) == (ro.nb_it, ro.nb_fev)
    assert rg.success == ro.success and rg.message == ro.message
    assert rel(rg.grad, ro.grad) < 1e-10
    assert rel(rg.stress, ro.stress) < 1e-10


def _variants(build, steps, tol, ntol):
    import scipy.fft as sfft
    out = []
    for lib in (sfft, None):
        saved = o._sfft
        o._sfft = lib
        try:
            cell = build()
            out.append(o.de_geus(cell, steps, o.SolverCG(cell, tol, 1000), ntol, 0.0, 0))
        finally:
            o._sfft = saved
    return out


def test_de_geus_3d_two_steps(mu):
    import test_gpu_parity as tp
    n = 15
    steps = []
    for k in (1, 2):
        D = np.zeros((3, 3))
        D[0, 0] = 0.01 * k
        D[0, 1] = D[1, 0] = 0.003 * k
        steps.append(D)
    tol, ntol = 1e-8, 1e-6
    ro, ro2 = _variants(lambda: tp._spheres_pair(mu, n, o.FINITE_STRAIN, 'le1')[0], steps, tol, ntol)
    gcell = tp._spheres_pair(mu, n, o.FINITE_STRAIN, 'le1')[1]
    rg = mu.solvers.de_geus(gcell, steps, mu.solvers.SolverCG(gcell, tol, 1000), ntol, 0.0)
    for a, b, b2 in zip(rg, ro, ro2):
        assert a.success and b.success
        assert a.nb_it == b.nb_it
        assert abs(a.nb_fev - b.nb_fev) <= max(1, 0.01 * b.nb_fev)
        assert rel(a.grad, b.grad) < 1e-10
        assert rel(a.stress, b.stress) < max(1e-10, 10 * rel(b2.stress, b.stress))


def test_de_geus_mixed_precision(mu):
    from muspectre_gb300 import workloads
    w = workloads.spheres(32, nsph=6)
    out = {}
    for prec in ('fp64', 'mixed'):
        cell = workloads.build_spheres_cell(mu, w, flags=mu.FFT_PlanFlags.estimate)
        r = mu.solvers.de_geus(cell, w['load'], mu.solvers.SolverCG(cell, 1e-8, 3000, precision=prec), 1e-8, 0.0)
        assert r.success, r.message
        out[prec] = cell.homogenised_stress()
    assert rel(out['mixed'], out['fp64']) < 1e-6
