"""Bounded waits of the TMA-fed passes, exercised without a GPU fault.

Every mbarrier wait of k_green_tma / k_last_inv_tma polls with a wall-clock limit;
when it runs out the kernel sets a device fault word and returns, and the host reads
the word after each FP32 CG solve.  musg_selftest_wait_timeout runs the same bounded
wait on an mbarrier that nothing completes (with a short limit): the host must see the
timeout, and the device must stay usable (a mixed-precision solve afterwards succeeds
and no stale fault is reported).
"""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def mu():
    import muspectre_gb300 as m
    if m.device_count() < 1:
        pytest.fail('no CUDA device visible')
    return m


def test_wait_times_out_and_device_stays_usable(mu):
    t0 = time.perf_counter()
    assert mu.selftest_wait_timeout(20.0)
    assert time.perf_counter() - t0 >= 0.02
    assert mu.selftest_wait_timeout(1.0)
    # the fault word was cleared: a TMA-path solve afterwards succeeds
    from muspectre_gb300 import workloads
    w = workloads.spheres(32, nsph=5, seed=4)
    cell = workloads.build_spheres_cell(mu, w, flags=mu.FFT_PlanFlags.estimate)
    r = mu.solvers.newton_cg(cell, w['load'], mu.solvers.SolverCG(cell, 1e-8, 2000, precision='mixed'), 1e-6, 0.0)
    assert r.success
    assert np.all(np.isfinite(cell.homogenised_stress()))


def test_wait_limit_is_checked(mu):
    with pytest.raises(Exception):
        mu.selftest_wait_timeout(0.0)
