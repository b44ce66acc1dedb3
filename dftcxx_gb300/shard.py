"""Grid Fock build split by atom cell over several ranks (GPUs or processes).

The reference builds one AtomicGrid per atom and sums the atoms' J blocks
(moleculargrid.cpp:193-261, 336-389); every quantity but three is local to a
fuzzy cell.  Here each rank holds whole cells, contiguous in atom order, and a
build is three local phases with one exchange after each:

  1. density on the rank's points      -> all-reduce of the integral of w rho
     (the correction factor of moleculargrid.cpp:132-146 needs the total)
  2. correction, LDA, rho_lm, Poisson,   -> all-gather of every cell's spline
     own-cell V, splines of its cells       data (cross-atom potential needs
                                            every other atom's U_lm splines)
  3. cross-atom V, J and XC on its points -> all-reduce of J, XC, E_xc, N, E_J

A backend is any object with ``density(P) -> float``, ``multipoles(total) ->
1-D float64 array`` (its cells' spline data, ``blob_per_cell`` doubles per
cell) and ``finish(blob_all, P) -> (J, XC, [E_xc, N, E_J])``; ``CellShard`` is
the CUDA one (dftg_create_cells / dftg_shard_*).  A communicator provides
``allreduce_sum`` and ``allgather`` over the backends of all ranks:
``TorchComm`` (torch.distributed, the backends of one rank per process, NCCL
or gloo) and
``InProcessComm`` (every backend in this process, run in lock-step phase by
phase; no device work waits on another rank's).
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import check
from .grid import MolecularGrid, _ptr


def partition_cells(natoms, nranks):
    """Contiguous, balanced blocks of atoms: [(first_cell, ncells)] per rank."""
    if nranks < 1 or nranks > natoms:
        raise ValueError("need 1 <= ranks <= atoms (%d ranks, %d atoms)" % (nranks, natoms))
    base, extra = divmod(natoms, nranks)
    out, first = [], 0
    for r in range(nranks):
        n = base + (1 if r < extra else 0)
        out.append((first, n))
        first += n
    return out


class CellShard(MolecularGrid):
    """The cells [first_cell, first_cell + ncells) of a molecule on one GPU."""

    def __init__(self, mol, radial_points, lebedev_order, lmax, first_cell, ncells, precision="fp64", device=0):
        super().__init__(mol, radial_points, lebedev_order, lmax, precision=precision, device=device,
                         cells=(first_cell, ncells))
        per, f, n = ctypes.c_size_t(), ctypes.c_int(), ctypes.c_int()
        check(_lib.load().dftg_shard_blob_size(self._h, ctypes.byref(per), ctypes.byref(f), ctypes.byref(n)))
        self.blob_per_cell = int(per.value)
        self.first_cell, self.ncells = int(f.value), int(n.value)

    def density(self, P):
        P = np.asfortranarray(P, dtype=np.float64)
        s = ctypes.c_double()
        check(_lib.load().dftg_shard_density(self._h, _ptr(P), ctypes.byref(s)))
        return s.value

    def multipoles(self, total):
        blob = np.zeros(self.blob_per_cell * self.ncells)
        check(_lib.load().dftg_shard_multipoles(self._h, float(total), _ptr(blob), blob.size))
        return blob

    def finish(self, blob_all, P=None):
        blob_all = np.ascontiguousarray(blob_all, dtype=np.float64)
        n = self.nbf
        J = np.zeros((n, n), order="F")
        XC = np.zeros((n, n), order="F")
        sc = np.zeros(3)
        check(_lib.load().dftg_shard_finish(self._h, _ptr(blob_all), blob_all.size, _ptr(J), _ptr(XC), _ptr(sc)))
        return np.ascontiguousarray(J), np.ascontiguousarray(XC), sc


class InProcessComm:
    """Every rank's backend in this process: sums and concatenations in rank order."""

    def allreduce_sum(self, parts):
        out = np.array(parts[0], dtype=np.float64, copy=True)
        for p in parts[1:]:
            out = out + p
        return out

    def allgather(self, parts):
        return np.concatenate([np.asarray(p, dtype=np.float64) for p in parts])


class TorchComm:
    """torch.distributed collectives, one backend per process.  Spline data is
    gathered as raw 64-bit words (the blobs hold split FP32 tables that must
    arrive bit for bit); ranks with fewer cells pad their block."""

    def __init__(self, device="cpu", group=None):
        import torch.distributed as dist
        self.dist = dist
        self.device = device
        self.group = group
        self.world = dist.get_world_size(group)

    def allreduce_sum(self, parts):
        import torch
        x = InProcessComm().allreduce_sum(parts)          # this process's shards first
        t = torch.from_numpy(np.ascontiguousarray(x, dtype=np.float64)).to(self.device)
        self.dist.all_reduce(t, group=self.group)
        return t.cpu().numpy()

    def allgather(self, parts):
        import torch
        x = InProcessComm().allgather(parts)
        words = np.ascontiguousarray(x, dtype=np.float64).view(np.int64)
        n = torch.tensor([words.size], dtype=torch.int64, device=self.device)
        sizes = [torch.zeros_like(n) for _ in range(self.world)]
        self.dist.all_gather(sizes, n, group=self.group)
        sizes = [int(v.item()) for v in sizes]
        buf = np.zeros(max(sizes), dtype=np.int64)
        buf[:words.size] = words
        t = torch.from_numpy(buf).to(self.device)
        outs = [torch.zeros_like(t) for _ in range(self.world)]
        self.dist.all_gather(outs, t, group=self.group)
        return np.concatenate([o.cpu().numpy()[:k] for o, k in zip(outs, sizes)]).view(np.float64)


def sharded_fock_build(P, shards, comm):
    """One grid Fock build of the molecule over the shards of all ranks.

    ``shards``: the backends this process holds (one under TorchComm, all of
    them under InProcessComm), in rank order.  Returns J, XC, E_xc, the
    integral of the corrected density and E_J of the whole molecule."""
    total = float(comm.allreduce_sum([np.array([s.density(P)]) for s in shards])[0])
    blob_all = comm.allgather([s.multipoles(total) for s in shards])
    fins = [s.finish(blob_all, P) for s in shards]
    n = fins[0][0].shape[0]
    tot = comm.allreduce_sum([np.concatenate([J.ravel(), X.ravel(), sc]) for J, X, sc in fins])
    J = tot[:n * n].reshape(n, n)
    XC = tot[n * n:2 * n * n].reshape(n, n)
    exc, nelec, ej = tot[2 * n * n:]
    return {"J": J, "XC": XC, "Exc": float(exc), "nelec": float(nelec), "EJ": float(ej), "total_wrho": total}
