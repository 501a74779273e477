"""Slab decomposition of the spectral grid over ranks: the layout and the exchanges of
the reference's distributed FFT engine (fftwmpi_engine.cc:40-242, FFTW-MPI with a
transposed output).

Real space is split along axis 0 into contiguous row blocks (FFTW's block size
ceil(n0 / world)).  After the transforms along the local axes, one all-to-all
transposes the distribution: k-space is split along axis 1 and axis 0 becomes local,
so the first-axis transform and the Green operator (pointwise in k) need no further
exchange; the inverse path transposes back.  A CG iteration additionally needs one
all-reduce of its scalars (communicator.hh:90-96).

This module moves data only (torch.distributed, any backend that has
all_to_all_single and all_reduce); the transforms and the operator are applied by the
caller on its local blocks.  One GPU holds every configuration of this project, so the
shipped multi-GPU mode runs independent replicas (muspectre_gb300.replicas); the slab
exchanges are exercised among CPU ranks.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import List, Tuple

import numpy as np


def block_bounds(n: int, world: int) -> List[Tuple[int, int]]:
    """[start, stop) of each rank's block of n entries (block ceil(n / world); the
    last ranks may hold fewer or none, as with fftw_mpi_local_size)."""
    b = int(math.ceil(n / world)) if n > 0 else 0
    return [(min(r * b, n), min((r + 1) * b, n)) for r in range(world)]


@dataclass
class SlabLayout:
    """Decomposition of a grid `res` (D = 2 or 3) over `world` ranks.  Spectral
    shape: res with the last axis halved to n/2 + 1; axis 1 of the spectrum is split
    after the transpose."""
    res: Tuple[int, ...]
    world: int
    rank: int

    def __post_init__(self):
        self.res = tuple(int(n) for n in self.res)
        self.spec = self.res[:-1] + (self.res[-1] // 2 + 1,)
        self.rows = block_bounds(self.res[0], self.world)     # real space, axis 0
        self.cols = block_bounds(self.spec[1], self.world)    # k-space, axis 1

    @property
    def local_rows(self):
        return self.rows[self.rank]

    @property
    def local_cols(self):
        return self.cols[self.rank]


def _as_real(t):
    import torch
    return torch.view_as_real(t.contiguous()) if t.is_complex() else t


def transpose_forward(block, layout: SlabLayout, group=None):
    """(nc, rows_r, n1, *rest) complex, split along axis 0 -> (nc, n0, cols_r, *rest),
    split along axis 1 (one all_to_all)."""
    import torch
    import torch.distributed as dist
    nc, m0 = block.shape[0], block.shape[1]
    rest = tuple(block.shape[3:])
    rsz = int(np.prod(rest)) if rest else 1
    chunks = [block[:, :, c0:c1].contiguous() for (c0, c1) in layout.cols]
    send = torch.cat([_as_real(c).reshape(-1) for c in chunks])
    in_splits = [nc * m0 * (c1 - c0) * rsz * 2 for (c0, c1) in layout.cols]
    c0, c1 = layout.local_cols
    w = c1 - c0
    out_splits = [nc * (r1 - r0) * w * rsz * 2 for (r0, r1) in layout.rows]
    recv = torch.empty(sum(out_splits), dtype=send.dtype)
    dist.all_to_all_single(recv, send, out_splits, in_splits, group=group)
    out = torch.empty((nc, layout.res[0], w) + rest, dtype=block.dtype)
    off = 0
    for (r0, r1), sz in zip(layout.rows, out_splits):
        part = recv[off:off + sz].reshape((nc, r1 - r0, w) + rest + (2,))
        out[:, r0:r1] = torch.view_as_complex(part.contiguous())
        off += sz
    return out


def transpose_backward(block, layout: SlabLayout, group=None):
    """Inverse of transpose_forward: (nc, n0, cols_r, *rest) -> (nc, rows_r, n1, *rest)."""
    import torch
    import torch.distributed as dist
    nc, w = block.shape[0], block.shape[2]
    rest = tuple(block.shape[3:])
    rsz = int(np.prod(rest)) if rest else 1
    chunks = [block[:, r0:r1].contiguous() for (r0, r1) in layout.rows]
    send = torch.cat([_as_real(c).reshape(-1) for c in chunks])
    in_splits = [nc * (r1 - r0) * w * rsz * 2 for (r0, r1) in layout.rows]
    r0, r1 = layout.local_rows
    m0 = r1 - r0
    out_splits = [nc * m0 * (c1 - c0) * rsz * 2 for (c0, c1) in layout.cols]
    recv = torch.empty(sum(out_splits), dtype=send.dtype)
    dist.all_to_all_single(recv, send, out_splits, in_splits, group=group)
    out = torch.empty((nc, m0, layout.spec[1]) + rest, dtype=block.dtype)
    off = 0
    for (c0, c1), sz in zip(layout.cols, out_splits):
        part = recv[off:off + sz].reshape((nc, m0, c1 - c0) + rest + (2,))
        out[:, :, c0:c1] = torch.view_as_complex(part.contiguous())
        off += sz
    return out


def allreduce_scalars(values, group=None):
    """Communicator::sum of a few FP64 scalars (communicator.hh:90-96)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor(list(values), dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return [float(v) for v in t]
