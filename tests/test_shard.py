"""Atom-cell sharded build (dftcxx_gb300.shard), checked on CPU ranks.

Each rank holds whole fuzzy cells and the ranks exchange three things per
build: the integral of w rho (all-reduce), every cell's spline data
(all-gather), and J, XC, E_xc, N, E_J (all-reduce).  The rank backends here are
the oracle's per-cell functions (oracle.OracleShard); the CUDA backend
(shard.CellShard) runs the same protocol in tests/test_gpu_shard.py.

Tolerances: the sharded J, XC, E_xc, N and E_J equal the single-process oracle
build to 1e-12 (only the order of the sums over cells changes)."""
import os
import tempfile

import numpy as np
import pytest

from dftcxx_gb300.molecule import Molecule, small_molecule
from dftcxx_gb300.shard import InProcessComm, partition_cells, sharded_fock_build

GRID = (16, 4, 6)


def _case():
    Z, xyz = small_molecule("NH3")
    mol = Molecule(Z, xyz, "sto3g")
    rng = np.random.default_rng(17)
    C = rng.normal(0, 0.3, size=(mol.nbf, mol.nelec // 2))
    return mol, C @ C.T


def _reference(oracle_mod, mol, P):
    g = oracle_mod.OracleGrid(mol, *GRID)
    r = g.fock_build(P)
    r["EJ"] = 2.0 * float(np.sum(P * r["J"]))
    return r


def _check(out, ref):
    assert np.abs(out["J"] - ref["J"]).max() <= 1e-12
    assert np.abs(out["XC"] - ref["XC"]).max() <= 1e-12
    assert abs(out["Exc"] - ref["Exc"]) <= 1e-12
    assert abs(out["nelec"] - ref["nelec"]) <= 1e-12
    assert abs(out["EJ"] - ref["EJ"]) <= 1e-12


def test_partition_cells():
    assert partition_cells(12, 5) == [(0, 3), (3, 3), (6, 2), (8, 2), (10, 2)]
    assert partition_cells(3, 3) == [(0, 1), (1, 1), (2, 1)]
    assert partition_cells(4, 1) == [(0, 4)]
    with pytest.raises(ValueError):
        partition_cells(2, 3)


@pytest.mark.parametrize("nranks", [1, 2, 4])
def test_sharded_oracle_in_process(oracle_mod, nranks):
    mol, P = _case()
    ref = _reference(oracle_mod, mol, P)
    shards = [oracle_mod.OracleShard(mol, *GRID, f, n) for f, n in partition_cells(mol.natoms, nranks)]
    _check(sharded_fock_build(P, shards, InProcessComm()), ref)


def _rank_main(rank, world, port, out_path):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from oracle import oracle
        from dftcxx_gb300.shard import TorchComm
        mol, P = _case()
        f, n = partition_cells(mol.natoms, world)[rank]
        out = sharded_fock_build(P, [oracle.OracleShard(mol, *GRID, f, n)], TorchComm())
        if rank == 0:
            np.savez(out_path, J=out["J"], XC=out["XC"], sc=np.array([out["Exc"], out["nelec"], out["EJ"]]))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_sharded_oracle_gloo_ranks(oracle_mod, world):
    """world processes, each with its cells only, exchanging over gloo."""
    import socket
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    mol, P = _case()
    ref = _reference(oracle_mod, mol, P)
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "out.npz")
        mp.start_processes(_rank_main, args=(world, port, path), nprocs=world, join=True, start_method="spawn")
        d = np.load(path)
        _check({"J": d["J"], "XC": d["XC"], "Exc": d["sc"][0], "nelec": d["sc"][1], "EJ": d["sc"][2]}, ref)
