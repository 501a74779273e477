"""Serving: requests of mixed size and load case run concurrently (lanes on
separate streams, requests of one kind batched, grids of different sizes in grouped
launches) and each result equals the same request solved alone: bit for bit when it
ran as a group of its own, within the mixed-precision bound (1e-6 relative
homogenised stress, the same Newton step count) when it shared a batch."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_same_alone_and_in_the_mix():
    import muspectre_gb300 as mu
    from muspectre_gb300 import serving
    if mu.device_count() < 1:
        pytest.fail('no CUDA device visible')
    reqs = [serving.c5_request(i, 100 + i, small=True) for i in range(6)]
    # duplicates of two requests (same shape) so that the server batches them
    for k, src in enumerate((1, 3)):
        r = serving.c5_request(6 + k, 100 + src, small=True)
        reqs.append(r)
    alone = {r.rid: serving.solve_alone(r) for r in reqs}
    budget = 3 * max(serving.estimate_bytes(r.res, r.formulation, any(m[0] == 'hep1' for m in r.materials),
                                            consistent=True) for r in reqs)
    srv = serving.Server(budget, lanes=3, max_batch=4)
    stats = serving.run_stream(reqs, rate_hz=0, server=srv)
    assert stats['requests'] == len(reqs)
    assert srv.peak_in_use <= budget
    for r in reqs:
        a, m = alone[r.rid], srv.results[r.rid]
        assert a.success == m.success
        if a.success:
            assert a.nb_it == m.nb_it
            tol = 1e-12 if m.batched_with == 1 else 1e-6
            assert np.linalg.norm(a.stress - m.stress) <= tol * np.linalg.norm(a.stress), (r.rid, m.batched_with)
    assert stats['p99_ms'] >= stats['p50_ms'] > 0


def _oracle_solve(o, req):
    """The request solved by the CPU oracle in FP64 (even grids with the extension)."""
    d = len(req.res)
    oc = o.Cell(req.res, [1.0] * d, int(req.formulation), allow_even=True)
    phase = np.asarray(req.phase).reshape(-1)
    line_search = False
    for k, (law, prm) in enumerate(req.materials):
        idx = np.flatnonzero(phase == k)
        if law == 'le1':
            m = o.MaterialLinearElastic1('m%d' % k, d, prm[0], prm[1])
        elif law == 'le4':
            m = o.MaterialLinearElastic4('m%d' % k, d)
            m.E, m.nu = np.asarray(prm[0]), np.asarray(prm[1])
        else:
            consistent = len(prm) > 4 and int(prm[4]) == 2
            line_search |= consistent
            m = o.MaterialHyperElastoPlastic1('m%d' % k, d, *prm[:4],
                                              tangent='consistent' if consistent else 'reference')
        m.pixels = list(idx)
        oc.add_material(m)
    rs = o.newton_cg(oc, req.steps, o.SolverCG(oc, 1e-8, 2000), 1e-6, 0.0, 0, line_search=line_search)
    return o.homogenised(rs[-1].stress, d)


def test_served_requests_vs_oracle():
    """Requests of the serving stream (small sizes) served in mixed precision, in the
    mix: homogenised stress within 1e-6 of the CPU oracle's FP64 solve."""
    import os

    import muspectre_gb300 as mu
    from muspectre_gb300 import serving
    from oracle import muspectre_oracle as o
    if mu.device_count() < 1:
        pytest.fail('no CUDA device visible')
    # seed 354 draws an elasto-plastic request (consistent tangent, 32^3, 3 load steps);
    # not every elasto-plastic draw converges (seed 334, compressive, stalls in CG in the
    # oracle's FP64 solve as well), so the sample is of requests the oracle solves
    reqs = [serving.c5_request(i, s, small=True) for i, s in enumerate((300, 301, 302, 303, 354))]
    srv = serving.Server(1 << 36, lanes=3, max_batch=4)
    serving.run_stream(reqs, rate_hz=0, server=srv)
    saved = o.FFT_WORKERS
    o.FFT_WORKERS = os.cpu_count() or 1
    try:
        for r in reqs:
            m = srv.results[r.rid]
            assert m.success, m.message
            ref = _oracle_solve(o, r)
            err = np.linalg.norm(m.stress - ref) / np.linalg.norm(ref)
            assert err < 1e-6, (r.rid, r.res, [x[0] for x in r.materials], err)
    finally:
        o.FFT_WORKERS = saved


def test_cancel_running_request():
    """A running solve stops at its next check when the server is asked to cancel the
    running groups: it completes unsolved ("cancelled while running") well before it
    would have finished, and the lane then solves the next request normally."""
    import time
    import muspectre_gb300 as mu
    from muspectre_gb300 import serving, workloads
    if mu.device_count() < 1:
        pytest.fail('no CUDA device visible')
    w = workloads.voronoi(n=64, nseeds=16, nsteps=20)
    mats = [('hep1', (w[p]['E'], w[p]['nu'], w[p]['tau_y0'], w[p]['H'], 2.0)) for p in ('A', 'B')]
    long_req = serving.Request(0, [64, 64, 64], int(mu.Formulation.finite_strain),
                               (~w['phaseA']).astype(np.uint8), mats, w['steps'])
    srv = serving.Server(1 << 36, lanes=1, max_batch=1)
    srv.submit(long_req)
    time.sleep(1.0)
    t0 = time.perf_counter()
    assert srv.cancel_running() == 1
    r = srv.result(0, timeout=60.0)
    assert not r.success and 'while running' in r.message, r.message
    assert time.perf_counter() - t0 < 10.0
    assert 0.5 < r.service < 20.0
    small = serving.c5_request(1, 101, small=True)
    srv.submit(small)
    srv.close()
    assert srv.result(1, timeout=120.0).success
