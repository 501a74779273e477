"""Batched solves: every cell of a batch gets exactly the results of a solo
newton_cg on it (the batched kernels run the same arithmetic per problem in the same
order), in FP64 and in mixed precision, and a failing cell leaves the others
untouched."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def mu():
    import muspectre_gb300 as m
    if m.device_count() < 1:
        pytest.fail('no CUDA device visible')
    return m


def _cells(mu, n, seeds, form='finite'):
    from muspectre_gb300 import workloads
    out = []
    for s in seeds:
        w = workloads.spheres(n, nsph=5, seed=s)
        out.append((workloads.build_spheres_cell(mu, w, flags=mu.FFT_PlanFlags.estimate), w))
    return out


# 24^3: generic passes; 32^3: register passes, where a solo mixed solve runs the
# TMA-fed Green and last-axis inverse kernels and a batched one the register Green
# kernel and the batched TMA inverse (same arithmetic, same reduction order)
@pytest.mark.parametrize('n', [24, 32])
@pytest.mark.parametrize('precision', ['fp64', 'mixed'])
def test_batch_equals_solo(mu, precision, n):
    cells = _cells(mu, n, [1, 2, 3])
    load = cells[0][1]['load']
    batch = mu.batch.BatchSolver([c for c, _ in cells], 1e-8, 2000, precision=precision)
    rb = batch.newton_cg(load, 1e-6, 0.0)
    for (c, w), res in zip(cells, rb):
        solo_cell = _cells(mu, n, [w['seed']])[0][0]
        rs = mu.solvers.newton_cg(solo_cell, load, mu.solvers.SolverCG(solo_cell, 1e-8, 2000, precision=precision),
                                  1e-6, 0.0)
        r = res[0]
        assert r.success and rs.success
        assert (r.nb_it, r.nb_fev) == (rs.nb_it, rs.nb_fev)
        assert np.array_equal(r.stress, rs.stress)
        assert np.array_equal(c.get_strain(), solo_cell.get_strain())


def test_batch_load_path_and_failure(mu):
    """Two load steps per cell with different loads; a cell given maxiter too small
    to converge is not part of this check -- instead one batch uses maxiter 1 and
    every cell reports the ConvergenceError message."""
    cells = _cells(mu, 16, [4, 5])
    loads = np.zeros((2, 2, 3, 3))
    loads[0, :, 0, 0] = [0.01, 0.02]
    loads[1, :, 1, 1] = [0.005, 0.01]
    rb = mu.batch.BatchSolver([c for c, _ in cells], 1e-8, 2000).newton_cg(loads, 1e-6, 0.0)
    for k, ((c, w), res) in enumerate(zip(cells, rb)):
        solo = _cells(mu, 16, [w['seed']])[0][0]
        rs = mu.solvers.newton_cg(solo, list(loads[k]), mu.solvers.SolverCG(solo, 1e-8, 2000), 1e-6, 0.0)
        for a, b in zip(res, rs):
            assert (a.nb_it, a.nb_fev) == (b.nb_it, b.nb_fev)
            assert np.array_equal(a.stress, b.stress)
    cells = _cells(mu, 16, [6, 7])
    rb = mu.batch.BatchSolver([c for c, _ in cells], 1e-8, 1).newton_cg(cells[0][1]['load'], 1e-6, 0.0)
    for res in rb:
        assert not res[0].success and 'not converged' in res[0].message


def _cell_n(mu, res, seed, form):
    """A two-phase LE1 cell of any grid (spheres of radii 0.1-0.25 of the shortest
    side), even axes with the extension."""
    rng = np.random.default_rng(seed)
    d = len(res)
    pts = np.stack(np.meshgrid(*[np.arange(n) for n in res], indexing='ij'), -1).reshape(-1, d).astype(float)
    inside = np.zeros(len(pts), dtype=bool)
    n = np.array(res, dtype=float)
    for _ in range(4):
        c = rng.uniform(0, 1, d) * n
        r = rng.uniform(0.1, 0.25) * n.min()
        dd = np.abs(pts - c)
        dd = np.minimum(dd, n - dd)
        inside |= (dd * dd).sum(1) < r * r
    cell = mu.Cell(res, [1.0] * d, form, allow_even=True)
    m = getattr(mu.material, 'MaterialLinearElastic1_%dd' % d)
    m.make(cell, 'incl', 210e9, .3).add_pixels(inside)
    m.make(cell, 'matrix', 3e9, .3).add_pixels(~inside)
    cell.initialise()
    return cell


# cells of different grids in one batch: grouped launches (each cell its own block
# range, FFT plans and sizes), power-of-two, 2/3/5-smooth and Bluestein lengths
UNEVEN = {
    'finite_3d': (0, [[16, 16, 16], [24, 20, 18], [15, 17, 12], [32, 16, 8]]),
    'small_3d': (1, [[16, 16, 16], [20, 24, 10]]),
    'finite_2d': (0, [[64, 64], [96, 50], [51, 51]]),
}


@pytest.mark.parametrize('case', sorted(UNEVEN))
@pytest.mark.parametrize('precision', ['fp64', 'mixed'])
def test_uneven_batch_matches_solo(mu, case, precision):
    """Each cell of an uneven batch against a solo newton_cg on the same cell: the
    same Newton step count; homogenised stress within 1e-8 in FP64 (both solves are
    the FP64 method; only the FFT kernels' rounding differs, which the CG can carry up
    to its tolerance into the stress of the last evaluation) and within 1e-6 in mixed
    precision (the metric's bound, the solo mixed solve running other FP32 kernels);
    the per-step homogenised stress of the result records equals the cell's."""
    form, grids = UNEVEN[case]
    d = len(grids[0])
    load = np.zeros((d, d))
    load[0, 0] = 0.01
    if form == 1:
        load[0, 1] = load[1, 0] = 0.003
    cells = [_cell_n(mu, g, 10 + k, form) for k, g in enumerate(grids)]
    rb = mu.batch.BatchSolver(cells, 1e-8, 3000, precision=precision).newton_cg(load, 1e-6, 0.0)
    tol = 1e-8 if precision == 'fp64' else 1e-6
    for k, (g, res) in enumerate(zip(grids, rb)):
        solo = _cell_n(mu, g, 10 + k, form)
        rs = mu.solvers.newton_cg(solo, load, mu.solvers.SolverCG(solo, 1e-8, 3000, precision=precision), 1e-6, 0.0)
        r = res[0]
        assert r.success and rs.success, (g, r.message, rs.message)
        assert r.nb_it == rs.nb_it
        hb = cells[k].homogenised_stress()
        hs = solo.homogenised_stress()
        assert np.linalg.norm(hb - hs) <= tol * np.linalg.norm(hs), (g, np.linalg.norm(hb - hs) / np.linalg.norm(hs))
        assert np.allclose(r.hom_stress, hb, rtol=0, atol=1e-12 * np.abs(hb).max())
