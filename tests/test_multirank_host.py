"""Multi-rank paths on CPU ranks (gloo), no GPU.

* Replicas (the shipped multi-GPU mode): round-robin sharding, and the whole-job
  throughput = all units / max time over ranks (muspectre_gb300.replicas, as
  bench.py reports it).
* Slab decomposition (the reference's distributed FFT engine, fftwmpi_engine.cc):
  each rank holds a block of rows, transforms its local axes, one all-to-all
  transposes to k-columns, the first-axis transform and the Green operator run on the
  local k-points, and the inverse path transposes back (muspectre_gb300.slab).  The
  projected field gathered from the ranks equals the single-rank projection of the
  oracle, and distributed dot products equal the global ones (the CG all-reduce).
"""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip('torch')
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _init(rank, world, port):
    dist.init_process_group('gloo', init_method='tcp://127.0.0.1:%d' % port, rank=rank, world_size=world)


def _replica_worker(rank, world, port, outdir):
    from muspectre_gb300 import replicas
    _init(rank, world, port)
    mine = replicas.shard(list(range(10)), rank, world)
    value, tmax, total = replicas.aggregate_throughput(len(mine), 1.0 + rank)
    np.save(os.path.join(outdir, 'rep%d.npy' % rank), np.array([len(mine), value, tmax, total]))
    dist.destroy_process_group()


@pytest.mark.parametrize('world', [2, 3])
def test_replicas_sharding_and_throughput(tmp_path, world):
    mp.spawn(_replica_worker, args=(world, _port(), str(tmp_path)), nprocs=world)
    rows = [np.load(tmp_path / ('rep%d.npy' % r)) for r in range(world)]
    assert sum(int(r[0]) for r in rows) == 10
    for r in rows:
        assert r[2] == float(world) and r[3] == 10.0
        assert abs(r[1] - 10.0 / world) < 1e-12


def _slab_worker(rank, world, port, res, kind, outdir):
    from muspectre_gb300 import slab
    from oracle import muspectre_oracle as o
    _init(rank, world, port)
    res = tuple(res)
    d = len(res)
    rng = np.random.default_rng(5)
    f = rng.standard_normal(res + (d, d))            # every rank draws the same field
    lay = slab.SlabLayout(res, world, rank)
    r0, r1 = lay.local_rows
    loc = f[r0:r1]
    # local axes: r2c along the last grid axis, c2c along the middle one(s)
    fh = np.fft.rfft(loc, axis=d - 1)
    for ax in range(1, d - 1):
        fh = np.fft.fft(fh, axis=ax)
    block = torch.from_numpy(np.ascontiguousarray(np.moveaxis(fh.reshape(fh.shape[:d] + (d * d,)), -1, 0)))
    t = slab.transpose_forward(block, lay).numpy()   # (nc, n0, cols, rest...)
    g = np.fft.fft(np.moveaxis(t, 0, -1), axis=0)    # (n0, cols, rest..., nc)
    c0, c1 = lay.local_cols
    proj = o.Projection(list(res), [1.0] * d, kind, allow_even=any(n % 2 == 0 for n in res))
    proj.xi = proj.xi[:, c0:c1]
    if proj.mask is not None:
        proj.mask = proj.mask[:, c0:c1]
    gh = proj._apply_hat(g.reshape(g.shape[:d] + (d, d))) if c1 > c0 else g.reshape(g.shape[:d] + (d, d))
    gi = np.fft.ifft(gh.reshape(g.shape), axis=0)
    back = slab.transpose_backward(torch.from_numpy(np.ascontiguousarray(np.moveaxis(gi, -1, 0))), lay).numpy()
    bh = np.moveaxis(back, 0, -1)
    for ax in range(1, d - 1):
        bh = np.fft.ifft(bh, axis=ax)
    out = np.fft.irfft(bh, n=res[-1], axis=d - 1).reshape(loc.shape)
    np.save(os.path.join(outdir, 'slab%d.npy' % rank), out)
    # distributed dot products (one all-reduce of the partial sums)
    dots = slab.allreduce_scalars([float(np.sum(out * out)), float(np.sum(out * loc))])
    np.save(os.path.join(outdir, 'dots%d.npy' % rank), np.array(dots))
    dist.destroy_process_group()


@pytest.mark.parametrize('res,kind,world', [
    ([9, 7], 'finite_fast', 2),
    ([7, 5, 9], 'small', 2),
    ([8, 6, 4], 'finite_fast', 2),
    ([5, 9, 7], 'finite_fast', 3),
])
def test_slab_projection_matches_single_rank(tmp_path, res, kind, world):
    from oracle import muspectre_oracle as o
    mp.spawn(_slab_worker, args=(world, _port(), res, kind, str(tmp_path)), nprocs=world)
    d = len(res)
    f = np.random.default_rng(5).standard_normal(tuple(res) + (d, d))
    proj = o.Projection(list(res), [1.0] * d, kind, allow_even=any(n % 2 == 0 for n in res))
    ref = o.t2_from_vec(proj.apply(o.t2_to_vec(f.reshape(-1, d, d))), d).reshape(f.shape)
    parts = [np.load(tmp_path / ('slab%d.npy' % r)) for r in range(world)]
    got = np.concatenate(parts, axis=0)
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
    dots = np.load(tmp_path / 'dots0.npy')
    assert abs(dots[0] - np.sum(ref * ref)) <= 1e-10 * np.sum(ref * ref)
    assert abs(dots[1] - np.sum(ref * f)) <= 1e-10 * abs(np.sum(ref * ref))


def test_block_bounds_cover_the_axis():
    from muspectre_gb300 import slab
    for n in (1, 5, 7, 8, 65):
        for w in (1, 2, 3, 4, 8):
            b = slab.block_bounds(n, w)
            assert len(b) == w and b[0][0] == 0 and b[-1][1] == n
            assert all(b[k][1] == b[k + 1][0] for k in range(w - 1))
