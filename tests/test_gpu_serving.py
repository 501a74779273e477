"""Serving: requests of mixed size and load case run concurrently (lanes on
separate streams, same-shape requests batched) and each result equals the same
request solved alone."""
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
    budget = 3 * max(serving.estimate_bytes(r.res, r.formulation, any(m[0] == 'hep1' for m in r.materials))
                     for r in reqs)
    srv = serving.Server(budget, lanes=3, max_batch=4)
    stats = serving.run_stream(reqs, rate_hz=0, server=srv)
    assert stats['requests'] == len(reqs)
    assert srv.peak_in_use <= budget
    for r in reqs:
        a, m = alone[r.rid], srv.results[r.rid]
        assert a.success == m.success
        if a.success:
            assert (a.nb_it, a.nb_fev) == (m.nb_it, m.nb_fev)
            assert np.linalg.norm(a.stress - m.stress) <= 1e-12 * np.linalg.norm(a.stress)
    assert stats['p99_ms'] >= stats['p50_ms'] > 0
