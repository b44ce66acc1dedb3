"""Atom-cell sharded build on the GPU (shard.CellShard over dftg_create_cells
and dftg_shard_*): the shards of a partition run one after another on one GPU
and exchange through InProcessComm (no device work waits on another shard's),
and the result must equal the single-context build.

Tolerances:
  FP64 shards vs FP64 single context   J, XC, E_xc, N, E_J within 1e-10
  mixed shards vs FP64 single context  the mixed bar: |dE_xc + dE_J| <= 1e-6 Ha,
                                       max|dJ|, max|dXC| <= 1e-6
"""
import numpy as np
import pytest

from dftcxx_gb300.molecule import Molecule, small_molecule

pytestmark = pytest.mark.gpu
GRID = (20, 7, 8)


def _case():
    Z, xyz = small_molecule("C6H6")
    mol = Molecule(Z, xyz, "p631")
    rng = np.random.default_rng(23)
    C = rng.normal(0, 0.2, size=(mol.nbf, mol.nelec // 2))
    return mol, C @ C.T


@pytest.fixture(scope="module")
def fp64_single(gpu_lib):
    from dftcxx_gb300.grid import MolecularGrid
    mol, P = _case()
    g = MolecularGrid(mol, *GRID, precision="fp64")
    r = g.fock_build(P)
    g.close()
    return r


@pytest.mark.parametrize("nranks", [2, 3, 12])
def test_fp64_shards_match_single_context(gpu_lib, fp64_single, nranks):
    from dftcxx_gb300.shard import CellShard, InProcessComm, partition_cells, sharded_fock_build
    mol, P = _case()
    shards = [CellShard(mol, *GRID, f, n, precision="fp64") for f, n in partition_cells(mol.natoms, nranks)]
    out = sharded_fock_build(P, shards, InProcessComm())
    ref = fp64_single
    assert np.abs(out["J"] - ref["J"]).max() <= 1e-10
    assert np.abs(out["XC"] - ref["XC"]).max() <= 1e-10
    assert abs(out["Exc"] - ref["Exc"]) <= 1e-10
    assert abs(out["nelec"] - ref["nelec"]) <= 1e-10
    assert abs(out["EJ"] - ref["EJ"]) <= 1e-10
    # a second build on the same shards (state is reset between builds)
    out2 = sharded_fock_build(P, shards, InProcessComm())
    assert np.abs(out2["J"] - out["J"]).max() <= 1e-14
    for s in shards:
        s.close()


def test_mixed_shards_within_the_mixed_bar(gpu_lib, fp64_single):
    from dftcxx_gb300.shard import CellShard, InProcessComm, partition_cells, sharded_fock_build
    mol, P = _case()
    shards = [CellShard(mol, *GRID, f, n, precision="mixed") for f, n in partition_cells(mol.natoms, 3)]
    out = sharded_fock_build(P, shards, InProcessComm())
    ref = fp64_single
    assert abs((out["Exc"] - ref["Exc"]) + (out["EJ"] - ref["EJ"])) <= 1e-6
    assert np.abs(out["J"] - ref["J"]).max() <= 1e-6
    assert np.abs(out["XC"] - ref["XC"]).max() <= 1e-6
    for s in shards:
        s.close()


def test_shard_context_rejects_whole_molecule_calls(gpu_lib):
    from dftcxx_gb300 import _lib
    from dftcxx_gb300.shard import CellShard
    mol, P = _case()
    s = CellShard(mol, *GRID, 0, 4, precision="fp64")
    with pytest.raises(_lib.DftgError) as e:
        s.fock_build(P)
    assert e.value.code == _lib.DFTG_ERR_STATE
    with pytest.raises(_lib.DftgError):
        s.multipoles(42.0)                 # out of order: no density yet
    s.close()
