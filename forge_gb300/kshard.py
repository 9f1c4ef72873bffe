"""k-point sharding of the SCF iteration across ranks (one GPU per rank).

The reference parallelises Solve over k with OpenMP threads and a reduction of zFockBulk
(HartreeFock.f90:424-478).  Across GPUs the same split needs exactly two exchanges per
iteration:
  1. all-gather of the numb x Nk window energies, so every rank sorts the same list and finds
     the same Fermi level, occupation counts and DegFactor (Main.f90:392-412);
  2. all-reduce (sum) of the local shares of P_new = (window + bulk)/Nk (Main.f90:506-511).
ODA, mixing and the potential are then computed redundantly on every rank.

The collective layer is any object with ``rank``, ``world``, ``allgather(np.ndarray) -> list`` and
``allreduce_sum(np.ndarray) -> np.ndarray`` (``TorchComm`` wraps torch.distributed: gloo on CPU,
NCCL between GPUs).  The per-rank compute is a worker with the methods used below;
``GpuShardWorker`` drives the CUDA library through its k-shard entry points.
"""
from __future__ import annotations

import ctypes as C
from typing import List, Sequence, Tuple

import numpy as np

from .api import HartreeFock, _check, _ptr


def partition(Nk: int, world: int) -> List[Tuple[int, int]]:
    """Contiguous, balanced flat-k ranges [k0, k1) per rank (uneven Nk is fine)."""
    base, extra = divmod(Nk, world)
    out, k = [], 0
    for r in range(world):
        n = base + (1 if r < extra else 0)
        out.append((k, k + n))
        k += n
    return out


class TorchComm:
    def __init__(self, dist=None):
        import torch.distributed as d
        self.d = dist or d
        self.rank = self.d.get_rank()
        self.world = self.d.get_world_size()

    def allgather(self, a: np.ndarray) -> list:
        import torch
        t = torch.from_numpy(np.ascontiguousarray(a))
        sizes = [torch.zeros(1, dtype=torch.int64) for _ in range(self.world)]
        self.d.all_gather(sizes, torch.tensor([t.numel()], dtype=torch.int64))
        m = int(max(s.item() for s in sizes))
        pad = torch.zeros(m, dtype=t.dtype)
        pad[:t.numel()] = t.reshape(-1)
        outs = [torch.zeros(m, dtype=t.dtype) for _ in range(self.world)]
        self.d.all_gather(outs, pad)
        return [o[:int(s.item())].numpy() for o, s in zip(outs, sizes)]

    def allreduce_sum(self, a: np.ndarray) -> np.ndarray:
        import torch
        t = torch.from_numpy(np.ascontiguousarray(a).view(np.float64).copy())
        self.d.all_reduce(t)
        return t.numpy().view(a.dtype).reshape(a.shape)


def sharded_iteration(worker, comm, energies: Sequence[float]):
    """One SCF iteration with k sharded over the ranks of `comm`; returns (step, energies, dn, residual)."""
    k0, k1 = partition(worker.Nk, comm.world)[comm.rank]
    local = worker.solve_local(k0, k1)                       # numb x (k1 - k0)
    parts = comm.allgather(local.T.reshape(-1))              # k-major pieces, in rank order
    bands = np.concatenate([p.reshape(-1, worker.numb) for p in parts], axis=0).T
    worker.set_global_bands(np.asfortranarray(bands))
    worker.fermi()
    P_local = worker.project_local()
    P_new = comm.allreduce_sum(P_local)
    return worker.step_and_mix(P_new, energies)


class GpuShardWorker:
    """Per-rank compute through the C-ABI k-shard entry points."""

    def __init__(self, hf: HartreeFock):
        self.hf = hf
        self.Nk, self.numb, self.N = hf.Nk, hf.numb, hf.N
        self._range = None

    def solve_local(self, k0, k1):
        if self._range != (k0, k1):
            _check(self.hf.lib.forge_gpu_set_kshard(self.hf.ctx, k0, k1))
            self._range = (k0, k1)
        B, _, _, _ = self.hf.Solve(None, None, bands=True)
        return np.asfortranarray(B[:, k0:k1])

    def set_global_bands(self, bands):
        _check(self.hf.lib.forge_gpu_set_bands(self.hf.ctx, _ptr(np.asfortranarray(bands, dtype=np.float64))))

    def fermi(self):
        return self.hf.FermiLevel()

    def project_local(self):
        P = np.zeros((self.N, self.N, 4), dtype=np.complex128, order="F")
        _check(self.hf.lib.forge_gpu_project_local(self.hf.ctx, _ptr(P)))
        return P

    def step_and_mix(self, P_new, energies):
        _check(self.hf.lib.forge_gpu_set_pnew(self.hf.ctx, _ptr(np.asfortranarray(P_new))))
        step, E = self.hf.OptimalStep(energies)
        dn, res = self.hf.MixPotential(step)
        return step, E, dn, res
