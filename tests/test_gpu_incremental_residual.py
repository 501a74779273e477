"""The mixed path's incremental Newton residual: one FP64 projection of G(-P) per load
step, then the FP32 projection of the previous residual minus the stress change since
(``SolverCG(..., incremental_residual=True)``, the mixed default).  Each case solves
the same cell three ways: FP64 (the plain method), mixed with every residual projected
in FP64, and mixed with the incremental residual.  The mixed paths return the stress
evaluated at the returned strain; the plain method returns the stress of its last
evaluation, one Newton increment behind its returned strain (solvers.cc:141-214), which
differs from the stress at that strain by up to ~1e-4 relative when the last increment
is just under newton_tol.  So the reference point is the FP64 run's stress evaluated at
its returned strain: both mixed results are within 1e-6 of it in homogenised stress, the
two mixed results within 1e-6 of each other, and the incremental one takes the same
Newton steps as the FP64-residual one or at most one more.  Cases: the 128^3 spheres
generator at 48^3 (finite strain LE1, the benchmarked formulation), a small-strain LE4
lognormal cell, a two-load-step LE1 ramp (the residual restarts in FP64 at each load
step), and a batch of two cells (the batched Newton loop keeps the same scheme, so the
batch equals its solo solves)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def mu():
    import muspectre_gb300 as m
    if m.device_count() < 1:
        pytest.fail('no CUDA device visible')
    return m


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b))


def _hom_at(cell, grad):
    """Homogenised stress evaluated at a returned strain field (history-free laws)."""
    d2 = cell.dim * cell.dim
    cell.evaluate_stress_tangent(np.asarray(grad).reshape(-1, d2).T)
    return cell.homogenised_stress()


def _three_ways(mu, make_cell, load, tol=1e-8, maxiter=2000, newton_tol=1e-6):
    out = {}
    for key, prec, inc in (('fp64', 'fp64', False), ('mixed_fp64res', 'mixed', False), ('mixed', 'mixed', True)):
        cell = make_cell()
        s = mu.solvers.SolverCG(cell, tol, maxiter, precision=prec, incremental_residual=inc)
        rs = mu.solvers.newton_cg(cell, load, s, newton_tol, 0.0, return_fields=(key == 'fp64'))
        rs = rs if isinstance(rs, list) else [rs]
        assert all(r.success for r in rs), (key, [r.message for r in rs])
        hom = [_hom_at(cell, r.grad) for r in rs] if key == 'fp64' else [r.hom_stress for r in rs]
        out[key] = (hom, [r.nb_it for r in rs])
    for k in range(len(out['fp64'][0])):
        ref = out['fp64'][0][k]
        assert rel(out['mixed'][0][k], ref) < 1e-6, (k, rel(out['mixed'][0][k], ref))
        assert rel(out['mixed_fp64res'][0][k], ref) < 1e-6, (k, rel(out['mixed_fp64res'][0][k], ref))
        assert rel(out['mixed'][0][k], out['mixed_fp64res'][0][k]) < 1e-6
        assert out['mixed_fp64res'][1][k] <= out['mixed'][1][k] <= out['mixed_fp64res'][1][k] + 1, \
            (out['mixed'][1], out['mixed_fp64res'][1])
    return out


def test_spheres48_finite_strain(mu):
    from muspectre_gb300 import workloads
    w = workloads.spheres(48)
    _three_ways(mu, lambda: workloads.build_spheres_cell(mu, w), w['load'], w['cg_tol'], w['maxiter'],
                w['newton_tol'])


def test_lognormal_le4_small_strain(mu):
    res = [32, 24, 40]
    n = int(np.prod(res))
    rng = np.random.default_rng(11)
    E = np.exp(rng.normal(np.log(1e9), 0.8, n))
    nu = rng.uniform(0.2, 0.4, n)

    def make():
        c = mu.Cell(res, [1., 1., 1.], mu.Formulation.small_strain, allow_even=True)
        mu.material.MaterialLinearElastic4_3d.make(c, 'm').add_pixels(np.arange(n), E, nu)
        c.initialise()
        return c
    load = np.zeros((3, 3))
    load[0, 1] = load[1, 0] = 0.01
    _three_ways(mu, make, load)


def test_two_load_steps(mu):
    from muspectre_gb300 import workloads
    w = workloads.spheres(32)
    load2 = [0.5 * w['load'], w['load']]
    _three_ways(mu, lambda: workloads.build_spheres_cell(mu, w), load2, w['cg_tol'], w['maxiter'], w['newton_tol'])


def test_batch_equals_solo(mu):
    from muspectre_gb300 import workloads, batch
    ws = [workloads.spheres(24, seed=5), workloads.spheres(24, seed=6)]
    solo = []
    for w in ws:
        cell = workloads.build_spheres_cell(mu, w)
        s = mu.solvers.SolverCG(cell, w['cg_tol'], w['maxiter'], precision='mixed')
        r = mu.solvers.newton_cg(cell, w['load'], s, w['newton_tol'], 0.0, return_fields=False)
        solo.append(r.hom_stress)
    cells = [workloads.build_spheres_cell(mu, w) for w in ws]
    bs = batch.BatchSolver(cells, ws[0]['cg_tol'], ws[0]['maxiter'], precision='mixed')
    res = bs.newton_cg(ws[0]['load'], ws[0]['newton_tol'], 0.0, return_stress=False)
    for b in range(2):
        assert res[b][0].success
        np.testing.assert_array_equal(res[b][0].hom_stress, solo[b])
