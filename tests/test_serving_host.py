"""Host logic of the native request server (no GPU: servers without lanes run
nothing): admission by HBM budget, batching by kind, memory returned on
completion, request validation, the config-5 request generator."""
import numpy as np

from muspectre_gb300 import serving
from muspectre_gb300._lib import CudaError
from muspectre_gb300.cell import Formulation


def _req(rid, n, hep=False):
    d = 2
    phase = np.zeros(n * n, dtype=np.int64)
    mats = [('hep1', (1e9, .3, 1e6, 1e7))] if hep else [('le1', (1e9, .3))]
    return serving.Request(rid, [n, n], int(Formulation.finite_strain), phase, mats, [np.eye(d) * 0.01])


def test_estimate_bytes_grows():
    a = serving.estimate_bytes([64, 64], Formulation.small_strain, False)
    b = serving.estimate_bytes([128, 128], Formulation.small_strain, False)
    c = serving.estimate_bytes([128, 128], Formulation.finite_strain, True)
    assert 0 < a < b < c
    assert serving.estimate_bytes([64] * 3, 0, False, 'fp64') != serving.estimate_bytes([64] * 3, 0, False, 'mixed')


def test_admission_budget_and_batching():
    """The native admission step (musg_server_admit on a server without lanes)."""
    fp = serving.estimate_bytes([64, 64], Formulation.finite_strain, False)
    srv = serving.Server(hbm_budget_bytes=int(2.5 * fp), lanes=0, max_batch=4)
    for rid, n in enumerate([64, 64, 96, 64, 64]):
        srv.submit(_req(rid, n))
    g1, used1 = srv._take()
    assert g1 == [0, 1]                           # same shape, two fit the budget
    assert srv.in_use == used1 <= srv.budget
    g2, used2 = srv._take()                       # 96^2 does not fit next to two 64^2
    assert g2 is None or srv.in_use <= srv.budget
    srv._release(used1)                           # first group completes
    g3, used3 = srv._take()
    assert g3 is not None and srv.in_use <= srv.budget
    assert srv.peak_in_use <= srv.budget


def test_oversized_request_refused():
    """A request larger than the whole HBM budget is refused at submission (it would
    overcommit the device even on an idle server); the server keeps serving."""
    import pytest
    fp = serving.estimate_bytes([64, 64], Formulation.finite_strain, False)
    srv = serving.Server(hbm_budget_bytes=fp, lanes=0)
    with pytest.raises(CudaError, match='budget'):
        srv.submit(_req(0, 96))
    srv.submit(_req(1, 64))
    g, used = srv._take()
    assert g == [1] and srv.in_use == used <= srv.budget
    assert srv._take()[0] is None


def test_batches_keep_kind_and_similar_size():
    """Requests of one kind (dimension, formulation, law kind, steps) share a batch,
    grids included that differ within a factor 8 in pixels; another law kind or a much
    larger grid waits for a batch of its own."""
    srv = serving.Server(hbm_budget_bytes=1 << 40, lanes=0, max_batch=8)
    srv.submit(_req(0, 64))
    srv.submit(_req(1, 64, hep=True))
    srv.submit(_req(2, 64))
    srv.submit(_req(3, 80))
    srv.submit(_req(4, 256))                        # 16x the pixels of 64^2
    g, _ = srv._take()
    assert g == [0, 2, 3]
    assert srv._take()[0] == [1]
    assert srv._take()[0] == [4]


def test_request_validation():
    import pytest
    srv = serving.Server(hbm_budget_bytes=1 << 30, lanes=0)
    bad = _req(0, 16)
    bad.phase = np.full(16 * 16, 3)               # material index beyond the list
    with pytest.raises(ValueError):
        srv.submit(bad)
    srv.close()
    with pytest.raises(RuntimeError):
        srv.submit(_req(1, 16))


def test_c5_generator_ranges():
    for seed in range(40):
        r = serving.c5_request(seed, seed, small=True)
        d = len(r.res)
        n = r.res[0]
        assert (d == 2 and 64 <= n <= 160) or (d == 3 and 32 <= n <= 40)
        assert serving._smooth235(n)
        if any(m[0] == 'hep1' for m in r.materials):
            assert r.formulation == Formulation.finite_strain
            assert 1 <= len(r.steps) <= 10
        for s in r.steps:
            assert np.allclose(s, s.T) and np.all(np.abs(s) <= 0.02 + 1e-12)


def test_stream_report_groups_failures_by_law():
    """run_stream's report: throughput over all requests and over the solved ones, and the
    failures grouped by the request's laws and the message's first sentence (a stand-in
    server; no GPU)."""
    reqs = [serving.c5_request(i, 2000 + i, small=True) for i in range(6)]

    class FakeServer:
        peak_in_use = 123
        admitted_batches = 1

        def __init__(self):
            self.results = {}

        def start(self):
            pass

        def submit(self, req):
            ok = req.rid % 3 != 0
            msg = '' if ok else 'Conjugate gradient has not converged. After 12 steps, the solver  FAILED'
            self.results[req.rid] = serving.Result(req.rid, ok, msg, 1, 10, np.zeros((2, 2)), 0.01)

        def close(self):
            pass

        def join(self):
            pass

    st = serving.run_stream(reqs, rate_hz=0.0, server=FakeServer())
    assert st['requests'] == 6 and st['succeeded'] == 4
    assert st['succeeded_per_s'] <= st['solves_per_s']
    assert sum(st['failed'].values()) == 2
    for key in st['failed']:
        law, msg = key.split(': ', 1)
        assert msg == 'Conjugate gradient has not converged.'
        assert set(law.split('+')) <= {'le1', 'le4', 'hep1'}
    assert st['peak_hbm_bytes'] == 123 and st['batches'] == 1


def test_cancel_waiting_requests():
    """Requests still waiting for admission are dropped on demand (a stream's
    deadline): each completes unsolved with its own message; admitted ones are not
    affected."""
    srv = serving.Server(hbm_budget_bytes=1 << 40, lanes=0, max_batch=1)
    for rid in range(3):
        srv.submit(_req(rid, 64))
    g, used = srv._take()
    assert g == [0] and srv.waiting() == 2
    assert srv.cancel_waiting() == 2 and srv.waiting() == 0
    for rid in (1, 2):
        r = srv.result(rid, timeout=1.0)
        assert not r.success and 'cancelled' in r.message
    assert srv._take()[0] is None


def test_cancel_running_without_lanes():
    """A server without lanes has no running group to stop."""
    srv = serving.Server(hbm_budget_bytes=1 << 40, lanes=0, max_batch=1)
    srv.submit(_req(0, 64))
    assert srv.cancel_running() == 0
    assert srv.waiting() == 1


def test_stream_window_ends_at_the_deadline():
    """run_stream with a deadline: nothing is submitted after it, the requests still
    waiting then are cancelled, and with stop_running the running groups are stopped
    too (a stand-in server that never finishes a request on its own; no GPU)."""
    import time
    reqs = [serving.c5_request(i, 3000 + i, small=True) for i in range(50)]

    class SlowServer:
        peak_in_use = 0
        admitted_batches = 0

        def __init__(self):
            self.results, self.queue, self.calls = {}, [], []

        def start(self):
            pass

        def submit(self, req):
            self.queue.append(req.rid)

        def close(self):
            pass

        def waiting(self):
            return len(self.queue) - 1  # one request "running", the rest waiting

        def cancel_waiting(self):
            self.calls.append('waiting')
            n = len(self.queue) - 1
            for rid in self.queue[1:]:
                self.results[rid] = serving.Result(rid, False, 'cancelled before admission', 0, 0,
                                                   np.zeros((2, 2)), 0.0)
            self.queue = self.queue[:1]
            return n

        def cancel_running(self):
            self.calls.append('running')
            rid = self.queue.pop()
            self.results[rid] = serving.Result(rid, False, 'cancelled while running', 0, 0, np.zeros((2, 2)), 0.0)
            return 1

        def join(self):
            assert not self.queue, 'a request would still be running'

    srv = SlowServer()
    t0 = time.perf_counter()
    st = serving.run_stream(reqs, rate_hz=100.0, server=srv, seed=3, deadline_s=0.2, stop_running=True)
    assert time.perf_counter() - t0 < 5.0
    assert 0 < st['offered'] < len(reqs)
    assert srv.calls == ['waiting', 'running']
    assert st['succeeded'] == 0 and st['cancelled'] == st['offered'] - 1
    assert sum(st['failed'].values()) == st['offered']
