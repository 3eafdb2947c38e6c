"""Replica fan-out over processes, one per GPU: the MSAMPI surface of the reference
(namsa/msa.py:994-1090) on torch.distributed.

The STEM scan shards by probe position with no exchange on the data path: every
process builds the same transmission stack and probe, simulates its own
contiguous block of positions, and the blocks are concatenated in position
order on rank 0.  The block split is the reference's (msa.py:1015-1022): each
rank takes n // world positions and the last rank also takes the remainder.
The reference scatters the position blocks from rank 0 and gathers the CBED
stacks with MPI Gatherv; here every rank derives the same position grid
locally and the gather is a padded torch.distributed.gather (NCCL with device
tensors, gloo with host tensors).
"""
from __future__ import annotations

import os
from datetime import timedelta

import numpy as np
import torch
import torch.distributed as dist

from .msa import MSAGPU


def block_parts(n, world):
    """[(start, stop)] per rank: n // world each, the last rank also the remainder."""
    part = n // world
    return [(r * part, n if r == world - 1 else (r + 1) * part) for r in range(world)]


def _device_for(group=None):
    backend = dist.get_backend(group)
    if backend == 'nccl':
        return torch.device('cuda', torch.cuda.current_device())
    return torch.device('cpu')


def gather_blocks(local, parts, dst=0, group=None):
    """Concatenate every rank's block (rank order = position order) on `dst`.

    local: this rank's array (rows = positions).  Blocks are padded to the
    largest block for the collective and trimmed after it.  Returns the full
    array on `dst`, None elsewhere.
    """
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    sizes = [b - a for a, b in parts]
    if len(parts) != world or local.shape[0] != sizes[rank]:
        raise ValueError(f'rank {rank}: block of {local.shape[0]} rows, expected {sizes[rank]} of {len(parts)} parts')
    dev = _device_for(group)
    tail = tuple(local.shape[1:])
    buf = torch.zeros((max(sizes),) + tail, dtype=torch.from_numpy(np.asarray(local)[:0]).dtype, device=dev)
    buf[:local.shape[0]] = torch.as_tensor(np.ascontiguousarray(local)).to(dev)
    bufs = [torch.empty_like(buf) for _ in range(world)] if rank == dst else None
    dist.gather(buf, bufs, dst=dst, group=group)
    if rank != dst:
        return None
    return np.concatenate([b[:s].cpu().numpy() for b, s in zip(bufs, sizes)])


def max_over_ranks(value, group=None):
    """The largest of every rank's `value` (a step time), on every rank."""
    t = torch.tensor([float(value)], dtype=torch.float64, device=_device_for(group))
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


def init_from_env(backend=None, timeout_s=300):
    """Process group from RANK / WORLD_SIZE / MASTER_ADDR / MASTER_PORT; NCCL when a GPU
    is visible, gloo otherwise.  With NCCL the process first selects GPU LOCAL_RANK
    (one process per GPU).  Returns (rank, world)."""
    if not dist.is_initialized():
        backend = backend or ('nccl' if torch.cuda.is_available() else 'gloo')
        if backend == 'nccl':
            torch.cuda.set_device(int(os.environ.get('LOCAL_RANK', 0)))
        dist.init_process_group(backend, init_method='env://', timeout=timedelta(seconds=timeout_s))
    return dist.get_rank(), dist.get_world_size()


class MSAReplicas(MSAGPU):
    """MSAGPU over one process per GPU (the reference's MSAMPI).

    The process group must be initialised (``init_from_env``).  After
    ``generate_probe_positions`` each rank keeps its block in
    ``probe_positions``; after ``multislice`` rank 0 holds the whole CBED stack
    in ``gathered`` (position order) and every rank its own block in ``probes``.
    """

    def __init__(self, *args, group=None, **kwargs):
        self.group = group
        self.rank, self.size = dist.get_rank(group), dist.get_world_size(group)
        super().__init__(*args, **kwargs)
        self.gathered = None

    def _partition(self):
        pos = np.asarray(self.probe_positions)
        self.total_num_probes = pos.shape[0]
        self.data_parts = block_parts(self.total_num_probes, self.size)
        a, b = self.data_parts[self.rank]
        self.all_probe_positions = pos
        self.probe_positions = pos[a:b]
        self.num_probes = np.int32(b - a)

    def generate_probe_positions(self, *args, **kwargs):
        super().generate_probe_positions(*args, **kwargs)
        self._partition()

    def set_probe_positions(self, positions):
        """Use an explicit (n, 2) [y, x] position list; each rank keeps its block."""
        self.probe_positions = np.asarray(positions, np.float32)
        self._partition()

    def multislice(self, *args, **kwargs):
        super().multislice(*args, **kwargs)
        self.gathered = gather_blocks(self.probes, self.data_parts, group=self.group)
        return None
