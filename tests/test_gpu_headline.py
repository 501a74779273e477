"""The benchmarked workloads' own kernel instantiations against the oracle.

The published throughput is produced by the 128³ finite-strain LE1 spheres cell with
autotuned launch shapes: the FP32 last-axis forward pass over rows of 128 with the
tangent rebuilt from F - I, the FP32 middle-axis pass over 128, the TMA-fed Green
pass over pencils of 128 (three components of a row per k-point), and the
bulk-copy-fed last-axis inverse.  The six-load-case small-strain LE4 workload runs the
same passes over length-256 axes with nine components.  Each test below builds those
exact shapes and checks them against the oracle: one application of the CG operator
G(K:dF) (cell_base.cc:150-192, projection_finite_strain_fast.cc:79-87,
projection_small_strain.cc:64-77) in FP32 (1e-5 relative) and FP64 (1e-12), and the
mixed-precision solve's homogenised stress against the FP64 solve (1e-6, the
metric's bound).  An odd twin of the headline grid (63³, where the reference method
applies without the even-grid extension) is solved in FP64 against the oracle.
"""
import os

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


@pytest.fixture()
def threaded_oracle():
    saved = o.FFT_WORKERS
    o.FFT_WORKERS = os.cpu_count() or 1
    yield o
    o.FFT_WORKERS = saved


def rel(a, b):
    a = np.asarray(a, dtype=float)
    b = np.asarray(b, dtype=float)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _perturbed_strain(n, d, finite, seed, amp=2e-3):
    rng = np.random.default_rng(seed)
    F = amp * rng.standard_normal((n, d, d))
    if finite:
        F[:, 0, 0] += 0.02
        F += np.eye(d)
    else:
        F = 0.5 * (F + F.transpose(0, 2, 1))
    return F, rng


def _operator_check(mu, gcell, ocell, finite, seed):
    d = gcell.dim
    n = gcell.nb_pixels
    F, rng = _perturbed_strain(n, d, finite, seed)
    ocell.F = o.t2_to_vec(F)
    ocell.evaluate_stress_tangent()
    gcell.evaluate_stress_tangent(o.t2_to_vec(F).reshape(n, -1).T)
    del F
    dF = rng.standard_normal(n * d * d)
    ref = ocell.directional_stiffness(dF)
    ocell.K = None  # the oracle's D^4 tangent is the largest array of the test
    dFa = dF.reshape(n, -1).T
    got64 = gcell.cg_operator(dFa, 'fp64').T.reshape(-1)
    got32 = gcell.cg_operator(dFa, 'mixed').T.reshape(-1)
    gds = gcell.directional_stiffness(dFa).T.reshape(-1)
    return rel(got64, ref), rel(got32, ref), rel(gds, ref)


def test_spheres128_operator_vs_oracle(mu, threaded_oracle):
    """The headline cell (128³, 40 spheres, autotuned shapes) at a perturbed
    finite-strain state: G(K:dF) from the FP32 CG kernels within 1e-5 of the oracle,
    from the FP64 CG kernels and from directional_stiffness within 1e-12."""
    from muspectre_gb300 import workloads
    w = workloads.spheres(128)
    gcell = workloads.build_spheres_cell(mu, w)
    ocell = workloads.build_spheres_oracle(o, w)
    # the solver's FP32 state (mixed-precision tangent planes) is what the bench uses
    mu.solvers.SolverCG(gcell, w['cg_tol'], w['maxiter'], precision='mixed')
    e64, e32, eds = _operator_check(mu, gcell, ocell, True, 128)
    assert e64 < 1e-12, e64
    assert eds < 1e-12, eds
    assert e32 < 1e-5, e32


def test_spheres128_mixed_solve_vs_fp64(mu):
    """The benchmarked solve: mixed-precision homogenised stress within 1e-6 of the
    FP64 solve of the same cell (the FP64 path itself is pinned to the oracle by the
    odd-twin test below and by the parity tests)."""
    from muspectre_gb300 import workloads
    w = workloads.spheres(128)
    cell = workloads.build_spheres_cell(mu, w)
    out = {}
    for prec in ('fp64', 'mixed'):
        s = mu.solvers.SolverCG(cell, w['cg_tol'], w['maxiter'], precision=prec)
        r = mu.solvers.newton_cg(cell, w['load'], s, w['newton_tol'], w['equil_tol'], return_fields=False)
        assert r.success, (prec, r.message)
        out[prec] = cell.homogenised_stress()
    assert rel(out['mixed'], out['fp64']) < 1e-6, rel(out['mixed'], out['fp64'])


def _lognormal_pair(mu, res, seed):
    rng = np.random.default_rng(seed)
    n = int(np.prod(res))
    E = np.exp(rng.normal(np.log(1e9), 0.8, n))
    nu = rng.uniform(0.2, 0.4, n)
    gcell = mu.Cell(res, [1., 1., 1.], mu.Formulation.small_strain, allow_even=True)
    mu.material.MaterialLinearElastic4_3d.make(gcell, 'm').add_pixels(np.arange(n), E, nu)
    gcell.initialise(mu.FFT_PlanFlags.measure)
    ocell = o.Cell(res, [1., 1., 1.], o.SMALL_STRAIN, allow_even=True)
    om = ocell.add_material(o.MaterialLinearElastic4('m', 3))
    om.pixels = list(range(n))
    om.E, om.nu = E, nu
    ocell.initialise()
    return gcell, ocell


@pytest.mark.parametrize('res', [[256, 32, 256], [32, 256, 256]])
def test_lognormal_le4_256_axes_operator_vs_oracle(mu, threaded_oracle, res):
    """The six-load-case workload's kernels: small-strain LE4 with per-pixel Lame
    planes, nine components, length-256 last axis and a length-256 Green axis
    ([256, 32, 256]) or middle axis ([32, 256, 256])."""
    gcell, ocell = _lognormal_pair(mu, res, 7)
    mu.solvers.SolverCG(gcell, 1e-7, 100, precision='mixed')
    e64, e32, eds = _operator_check(mu, gcell, ocell, False, 256)
    assert e64 < 1e-12, e64
    assert eds < 1e-12, eds
    assert e32 < 1e-5, e32


def test_lognormal_le4_256_axes_mixed_solve(mu):
    """One unit load case of the six-load-case workload on a [256, 32, 256] grid:
    mixed-precision homogenised stress within 1e-6 of the FP64 solve."""
    res = [256, 32, 256]
    out = {}
    load = np.zeros((3, 3))
    load[0, 1] = load[1, 0] = 0.5
    for prec in ('fp64', 'mixed'):
        gcell, _ = _lognormal_pair(mu, res, 7) if prec == 'fp64' else (out['cell'], None)
        out['cell'] = gcell
        s = mu.solvers.SolverCG(gcell, 1e-7, 4000, precision=prec)
        r = mu.solvers.newton_cg(gcell, load, s, 1e-6, 0.0, return_fields=False)
        assert r.success, (prec, r.message)
        out[prec] = gcell.homogenised_stress()
    assert rel(out['mixed'], out['fp64']) < 1e-6, rel(out['mixed'], out['fp64'])


def test_odd_twin_63_fp64_vs_oracle(mu, threaded_oracle):
    """The headline generator on the odd 63³ grid (40 spheres with radii scaled by
    63/128, no even-grid extension), solved in FP64 on the GPU and by the oracle:
    the same Newton step count, CG counts within 1%, strain field and homogenised
    strain to 1e-10, homogenised stress to 1e-10 (or within 10x the oracle's own
    scipy-vs-numpy FFT spread where the returned stress carries the CG tolerance)."""
    from muspectre_gb300 import workloads
    w = workloads.spheres(63)
    gcell = workloads.build_spheres_cell(mu, w, allow_even=False)
    ocell = workloads.build_spheres_oracle(o, w, allow_even=False)
    ro = o.newton_cg(ocell, w['load'], o.SolverCG(ocell, w['cg_tol'], w['maxiter']), w['newton_tol'],
                     w['equil_tol'], 0)
    rg = mu.solvers.newton_cg(gcell, w['load'], mu.solvers.SolverCG(gcell, w['cg_tol'], w['maxiter']),
                              w['newton_tol'], w['equil_tol'])
    assert rg.success and ro.success
    assert rg.nb_it == ro.nb_it
    assert abs(rg.nb_fev - ro.nb_fev) <= max(1, 0.01 * ro.nb_fev), (rg.nb_fev, ro.nb_fev)
    assert rel(rg.grad, ro.grad) < 1e-10
    assert rel(o.homogenised(rg.grad, 3), o.homogenised(ro.grad, 3)) < 1e-10
    err = rel(o.homogenised(rg.stress, 3), o.homogenised(ro.stress, 3))
    if err >= 1e-10:
        saved = o._sfft
        o._sfft = None
        try:
            oc2 = workloads.build_spheres_oracle(o, w, allow_even=False)
            r2 = o.newton_cg(oc2, w['load'], o.SolverCG(oc2, w['cg_tol'], w['maxiter']), w['newton_tol'],
                             w['equil_tol'], 0)
        finally:
            o._sfft = saved
        spread = rel(o.homogenised(r2.stress, 3), o.homogenised(ro.stress, 3))
        assert err < 10 * spread, (err, spread)
