"""Continuous-batching request server: the Python face of musg_server_* (include/musg.h).

Requests (one RVE each: grid, formulation, microstructure, load path) arrive over
time.  The native server admits a request when a lane is free and its estimated
device footprint fits the HBM budget next to everything already admitted; waiting
requests of the same kind (dimension, formulation, law kind, load steps; grids within
a factor 8 in pixels) are taken together and solved as one batch (one launch per CG
pass for all of them, grouped over different grids).  Each lane is a native host thread with its own CUDA
stream, so admitted requests overlap on the device.  Fields and plastic state stay on
the device for all load steps of a request; memory returns to the budget when the
request completes.  Latency = completion - submission.

A request batched with requests of its own grid is computed by the kernels of its
solo solve in the same order (per-request reductions in a fixed order), so its result
is the same bit for bit; batched with other grids it runs the generic pass kernels
and its result equals the solo one within rounding (``tests/test_gpu_serving.py``).
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass
from typing import Dict, List, Optional

import numpy as np

from . import _lib as L
from .cell import Formulation

_LAWS = {'le1': L.LAW_LE1, 'le2': L.LAW_LE2, 'le3': L.LAW_LE3, 'le4': L.LAW_LE4, 'hep1': L.LAW_HEP1}
_PREC = {'fp64': L.PRECISION_FP64, 'mixed': L.PRECISION_MIXED}


@dataclass
class Request:
    """One homogenization solve.  ``phase``: material index per pixel (row-major);
    ``materials``: per index (law, params) with law 'le1' (E, nu), 'le4' (per-pixel
    arrays E, nu over the phase's pixels) or 'hep1' (E, nu, tau_y0, H)."""
    rid: int
    res: List[int]
    formulation: int
    phase: np.ndarray
    materials: List[tuple]
    steps: List[np.ndarray]
    arrival: float = 0.0
    lengths: Optional[List[float]] = None

    def shape_key(self):
        kinds = tuple(sorted({m[0] == 'hep1' for m in self.materials}))
        return (tuple(self.res), int(self.formulation), kinds, len(self.steps))


@dataclass
class Result:
    rid: int
    success: bool
    message: str
    nb_it: int
    nb_fev: int
    stress: np.ndarray          # homogenised PK1 / Cauchy stress of the last step (D×D)
    latency: float
    batched_with: int = 1
    service: float = 0.0        # admission -> completion (seconds)


def _native(req):
    """musg_request for req, and the arrays it points into (kept alive by the caller)."""
    d = len(req.res)
    npx = int(np.prod(req.res))
    nm = len(req.materials)
    laws = np.array([_LAWS[m[0]] for m in req.materials], dtype=np.int32)
    params = np.zeros((nm, 5))
    phase = np.ascontiguousarray(np.asarray(req.phase).reshape(-1), dtype=np.uint8)
    per_pixel = None
    for k, (law, prm) in enumerate(req.materials):
        if law == 'le4' or law == 'le3':
            if per_pixel is None:
                per_pixel = np.zeros((npx, 2))
            idx = np.flatnonzero(phase == k)
            per_pixel[idx, 0] = np.asarray(prm[0], dtype=np.float64).reshape(-1)
            per_pixel[idx, 1] = np.asarray(prm[1], dtype=np.float64).reshape(-1)
        else:
            params[k, :len(prm)] = prm
    steps = np.ascontiguousarray(np.stack([np.asarray(s, dtype=np.float64).T.reshape(-1) for s in req.steps]))
    r = L.Request()
    r.dim = d
    for i in range(d):
        r.resolutions[i] = int(req.res[i])
        r.lengths[i] = float((req.lengths or [1.0] * d)[i])
    r.formulation = int(req.formulation)
    r.flags = L.FLAG_ALLOW_EVEN
    r.nb_materials = nm
    r.laws = laws.ctypes.data_as(C.POINTER(C.c_int))
    r.params = params.ctypes.data_as(C.POINTER(C.c_double))
    r.phase = phase.ctypes.data_as(C.POINTER(C.c_ubyte))
    if per_pixel is not None:
        r.per_pixel = per_pixel.ctypes.data_as(C.POINTER(C.c_double))
        r.per_pixel_stride = 2
    r.nb_steps = len(req.steps)
    r.load_steps = steps.ctypes.data_as(C.POINTER(C.c_double))
    return r, (laws, params, phase, per_pixel, steps)


def estimate_bytes(res, formulation, has_hep, precision='mixed', consistent=False):
    """Device memory of one admitted request (fields, spectra, tangent data, CG
    vectors, state), as the library allocates it (musg_request_bytes);
    ``consistent``: its elasto-plastic material has the consistent tangent."""
    r = L.Request()
    r.dim = len(res)
    for i, n in enumerate(res):
        r.resolutions[i] = int(n)
    r.formulation = int(formulation)
    r.nb_materials = 1
    law = (C.c_int * 1)(L.LAW_HEP1 if has_hep else L.LAW_LE1)
    r.laws = C.cast(law, C.POINTER(C.c_int))
    prm = (C.c_double * 5)(0, 0, 0, 0, 2.0 if consistent else 0.0)
    r.params = C.cast(prm, C.POINTER(C.c_double))
    out = C.c_ulonglong(0)
    L.check(L.lib().musg_request_bytes(C.byref(r), _PREC[precision], C.byref(out)))
    return int(out.value)


class Server:
    """Admission by HBM budget, native lanes on separate streams, batching by kind.
    ``lanes=0`` runs nothing: ``_take`` / ``_release`` then step the admission by
    hand (host-side checks of the policy)."""

    def __init__(self, hbm_budget_bytes, lanes=4, max_batch=8, precision='mixed', tol=1e-8, maxiter=2000,
                 newton_tol=1e-6):
        self.budget = int(hbm_budget_bytes)
        self.lanes = int(lanes)
        self.max_batch = int(max_batch)
        self.precision = precision
        self.results: Dict[int, Result] = {}
        self._ids: Dict[int, tuple] = {}
        self._by_id: Dict[int, int] = {}
        h = C.c_void_p()
        L.check(L.lib().musg_server_create(C.c_ulonglong(self.budget), self.lanes, self.max_batch, _PREC[precision],
                                           float(tol), int(maxiter), float(newton_tol), C.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, '_h', None)
        if h is not None and h.value:
            try:
                L.lib().musg_server_destroy(h)
            except Exception:
                pass
            self._h = None

    # ------------------------------------------------------------------ client side
    def submit(self, req: Request):
        req.arrival = time.perf_counter()
        r, keep = _native(req)
        nid = C.c_longlong(0)
        L.check(L.lib().musg_server_submit(self._h, C.byref(r), C.byref(nid)))
        self._ids[req.rid] = (int(nid.value), len(req.res))
        self._by_id[int(nid.value)] = req.rid
        return req.rid

    def close(self):
        L.check(L.lib().musg_server_close(self._h))

    def cancel_waiting(self):
        """Drop the requests not yet admitted (they complete unsolved); returns their number."""
        n = C.c_longlong(0)
        L.check(L.lib().musg_server_cancel_waiting(self._h, C.byref(n)))
        return int(n.value)

    def cancel_running(self):
        """Stop the groups being solved at their next check (they complete unsolved,
        "cancelled while running"); returns the number of groups signalled."""
        n = C.c_longlong(0)
        L.check(L.lib().musg_server_cancel_running(self._h, C.byref(n)))
        return int(n.value)

    def start(self):
        """Lanes start with the server; kept for the call sequence of run_stream."""

    def result(self, rid, timeout=3600.0):
        if rid in self.results:
            return self.results[rid]
        nid, d = self._ids[rid]
        out = L.ServerResult()
        L.check(L.lib().musg_server_wait(self._h, nid, float(timeout), C.byref(out)))
        stress = np.array(out.stress[:d * d]).reshape(d, d).T
        res = Result(rid, bool(out.success), out.message.decode('utf-8', 'replace'), int(out.nb_it), int(out.nb_fev),
                     stress if out.success else np.full((d, d), np.nan), float(out.latency_s),
                     int(out.batched_with), float(out.service_s))
        self.results[rid] = res
        return res

    def join(self, timeout=3600.0):
        for rid in list(self._ids):
            self.result(rid, timeout)

    def _stats(self):
        st = L.ServerStats()
        L.check(L.lib().musg_server_get_stats(self._h, C.byref(st)))
        return st

    @property
    def in_use(self):
        return int(self._stats().in_use)

    @property
    def peak_in_use(self):
        return int(self._stats().peak_in_use)

    @property
    def admitted_batches(self):
        return int(self._stats().batches)

    def waiting(self):
        """Requests submitted and not yet admitted."""
        return int(self._stats().queued)

    # ------------------------------------------------------------------ admission by hand
    def _take(self):
        """One admission step (servers without lanes): (rids of the group, bytes)."""
        ids = (C.c_longlong * self.max_batch)()
        n = C.c_int(0)
        used = C.c_ulonglong(0)
        L.check(L.lib().musg_server_admit(self._h, ids, self.max_batch, C.byref(n), C.byref(used)))
        if n.value == 0:
            return None, 0
        return [self._by_id[int(ids[k])] for k in range(n.value)], int(used.value)

    def _release(self, used):
        L.check(L.lib().musg_server_release(self._h, C.c_ulonglong(int(used))))


def solve_alone(req, tol=1e-8, maxiter=2000, newton_tol=1e-6, precision='mixed', timeout_s=None):
    """The reference point of the serving test: the request on its own (one lane,
    no batching, nothing else running).  With ``timeout_s`` a solve still running
    then is cancelled (its result is unsolved, "cancelled while running")."""
    srv = Server(1 << 62, lanes=1, max_batch=1, precision=precision, tol=tol, maxiter=maxiter, newton_tol=newton_tol)
    srv.submit(req)
    srv.close()
    if timeout_s is not None:
        try:
            return srv.result(req.rid, float(timeout_s))
        except RuntimeError:
            srv.cancel_running()
    return srv.result(req.rid)


def c5_request(rid, seed, small=False):
    """A request of the mixed serving stream, drawn from its own seed: 2-D (64..1024, 2/3/5-smooth)
    or 3-D (32..160, 2/3/5-smooth); small or finite strain; LE1/LE4, or HEP1 with 1-10
    load steps (finite strain only; the consistent tangent, so that heterogeneous
    cells converge); 1-60 spheres; E ~ U[1e9, 300e9], nu ~ U[0.2, 0.4]; symmetric
    macro strain entries ~ U[-0.02, 0.02].  ``small`` caps the sizes (tests)."""
    rng = np.random.default_rng(seed)
    smooth = lambda lo, hi: [n for n in range(lo, hi + 1) if _smooth235(n)]
    d = 2 if rng.random() < 0.5 else 3
    if d == 2:
        sizes = smooth(64, 160 if small else 1024)
    else:
        sizes = smooth(32, 40 if small else 160)
    n = int(rng.choice(sizes))
    res = [n] * d
    hep = rng.random() < 0.2
    form = Formulation.finite_strain if (hep or rng.random() < 0.5) else Formulation.small_strain
    nsph = int(rng.integers(1, 61))
    inside = np.zeros([n] * d, dtype=bool)
    for _ in range(nsph):
        c = rng.uniform(0, n, d)
        r = rng.uniform(0.03, 0.15) * n
        # the sphere's periodic bounding box only (minimum-image distance per axis)
        idx, dist2 = [], 0.0
        for a in range(d):
            lo, hi = int(np.floor(c[a] - r)), int(np.ceil(c[a] + r))
            ii = np.arange(lo, hi + 1)
            da = np.abs(ii - c[a])
            da = np.minimum(da, n - da)
            shape = [1] * d
            shape[a] = ii.size
            idx.append(np.mod(ii, n))
            dist2 = dist2 + (da * da).reshape(shape)
        inside[np.ix_(*idx)] |= dist2 < r * r
    phase = inside.reshape(-1).astype(np.uint8)
    mats = []
    for k in range(2):
        E, nu = float(rng.uniform(1e9, 300e9)), float(rng.uniform(0.2, 0.4))
        if hep:
            # the consistent tangent (mode 2), solved with newton_cg's line search
            mats.append(('hep1', (E, nu, E * 1e-3, E * 5e-3, 2.0)))
        elif rng.random() < 0.5:
            mats.append(('le1', (E, nu)))
        else:
            cnt = int((phase == k).sum())
            mats.append(('le4', (rng.uniform(0.5, 1.5, cnt) * E, np.full(cnt, nu))))
    eps = rng.uniform(-0.02, 0.02, (d, d))
    eps = 0.5 * (eps + eps.T)
    nsteps = int(rng.integers(1, 11)) if hep else 1
    steps = [eps * (k + 1) / nsteps for k in range(nsteps)]
    return Request(rid, res, int(form), phase, mats, steps)


def _smooth235(n):
    for p in (2, 3, 5):
        while n % p == 0:
            n //= p
    return n == 1


def run_stream(requests, rate_hz, server, seed=12345, deadline_s=None, stop_running=False):
    """Feed requests open loop with Poisson arrivals (exponential gaps at rate_hz;
    rate_hz <= 0 submits them all at once), wait for all.  A request the server
    refuses at submission (larger than the HBM budget, invalid) counts as failed.
    With ``deadline_s``, no request is submitted later than that after the first
    submission, and the requests still waiting for admission then are cancelled
    (counted as not completed; ``offered`` counts the submitted ones); with
    ``stop_running`` the groups still being solved then are stopped too, so the
    stream ends at the deadline (a measurement window).  Throughput is succeeded
    requests over the wall time from the first submission to the last completion."""
    rng = np.random.default_rng(seed)
    server.start()
    refused = {}
    t0 = time.perf_counter()
    next_t = t0
    offered = 0
    for req in requests:
        if rate_hz > 0:
            now = time.perf_counter()
            if next_t > now:
                time.sleep(next_t - now)
            next_t += float(rng.exponential(1.0 / rate_hz))
        if deadline_s is not None and time.perf_counter() - t0 > deadline_s:
            break
        offered += 1
        try:
            server.submit(req)
        except (L.CudaError, ValueError, RuntimeError) as e:
            refused[req.rid] = str(e)[:60]
    server.close()
    cancelled = 0
    if deadline_s is not None:
        while time.perf_counter() - t0 < deadline_s and server.waiting() > 0:
            time.sleep(0.05)
        cancelled = server.cancel_waiting()
        if stop_running:
            server.cancel_running()
    server.join()
    wall = time.perf_counter() - t0
    res = server.results
    lat = np.array([r.latency for r in res.values()]) if res else np.zeros(1)
    ok = sum(r.success for r in res.values())
    laws = {req.rid: '+'.join(sorted({m[0] for m in req.materials})) for req in requests}
    failed = {}
    for rid, r in res.items():
        if not r.success:
            key = '%s: %s' % (laws.get(rid, '?'), r.message.split(' After ')[0][:60])
            failed[key] = failed.get(key, 0) + 1
    for rid, msg in refused.items():
        key = '%s: refused: %s' % (laws.get(rid, '?'), msg)
        failed[key] = failed.get(key, 0) + 1
    ok_lat = np.array([r.latency for r in res.values() if r.success]) if ok else np.zeros(1)
    return {'requests': len(requests), 'offered': offered, 'succeeded': int(ok), 'refused': len(refused),
            'cancelled': cancelled, 'wall_s': wall,
            'offered_rate_hz': float(rate_hz) if rate_hz > 0 else None,
            'solves_per_s': offered / wall, 'succeeded_per_s': int(ok) / wall, 'failed': failed,
            'p50_ms': float(np.percentile(lat, 50) * 1e3), 'p99_ms': float(np.percentile(lat, 99) * 1e3),
            'p50_ms_succeeded': float(np.percentile(ok_lat, 50) * 1e3),
            'p99_ms_succeeded': float(np.percentile(ok_lat, 99) * 1e3),
            'peak_hbm_bytes': server.peak_in_use, 'batches': server.admitted_batches}
