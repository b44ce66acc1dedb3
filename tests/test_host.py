"""Host-side logic without a GPU: input files, basis ordering and counts,
settings presets, geometries, and the rank reduction of the benchmark
(two gloo ranks on the CPU)."""
import math
import os
import socket

import numpy as np
import pytest

from dftcxx_gb300 import molecule as M


def test_basis_sizes_of_the_workloads():
    Z, xyz = M.h2o()
    assert M.Molecule(Z, xyz, "sto3g").nbf == 7
    Z, xyz = M.benzene()
    mol = M.Molecule(Z, xyz, "p631")
    assert mol.nbf == 66 and mol.natoms == 12 and mol.nelec == 42
    for n in range(2, 11):
        Z, xyz = M.alkane(n)
        mol = M.Molecule(Z, xyz, "p631")
        assert mol.natoms == 3 * n + 2
        assert mol.nbf == 13 * n + 4


def test_basis_functions_ordered_by_element_then_atom():
    # molecule.cpp:135-238: elements in increasing Z, atoms in input order,
    # P shells as (x, y, z)
    Z, xyz = M.h2o()
    mol = M.Molecule(Z, xyz, "sto3g")
    assert list(mol.bf_atom) == [1, 2, 0, 0, 0, 0, 0]
    lmn = np.asarray(mol.bf_lmn).reshape(-1, 3)
    assert [tuple(r) for r in lmn[4:]] == [(1, 0, 0), (0, 1, 0), (0, 0, 1)]


def test_geometries():
    Z, xyz = M.benzene()
    xyz = np.asarray(xyz)
    r = np.linalg.norm(xyz, axis=1)
    assert np.allclose(r[:6], 2.640) and np.allclose(r[6:], 4.680)
    assert np.allclose(np.linalg.norm(xyz[0] - xyz[1]), 2.640)
    Z, xyz = M.alkane(4)
    xyz = np.asarray(xyz)
    C = xyz[:4]
    assert np.allclose(np.linalg.norm(np.diff(C, axis=0), axis=1), 2.910)
    d = np.linalg.norm(xyz[4:, None, :] - C[None, :, :], axis=2).min(axis=1)
    assert np.allclose(d, 2.060)
    v1, v2 = C[0] - C[1], C[2] - C[1]
    ang = math.degrees(math.acos(v1 @ v2 / np.linalg.norm(v1) / np.linalg.norm(v2)))
    assert abs(ang - 109.4712) < 1e-3


def test_settings_presets_and_overrides():
    s = M.Settings()
    assert (s.radial_points, s.lebedev_order, s.lmax) == (15, 7, 8)
    s = M.Settings({"grid": "fine", "lmax": "12", "radial_points": "x"})
    assert (s.radial_points, s.lebedev_order, s.lmax) == (20, 8, 12)
    assert M.Settings({"hartree_evaluation": "two_electron_integrals"}).hartree_evaluation == "two_electron_integrals"
    assert M.Settings({"hartree_evaluation": "other"}).hartree_evaluation == "becke_grid"
    assert M.LEBEDEV_NPTS[M.LEBEDEV_302] == 302


def test_read_input_file(tmp_path):
    p = tmp_path / "mol.in"
    p.write_text("name = test water\nbasis = sto3g\nunits = angstrom\ngrid = coarse\n\nsystem:\n3\n"
                 "O 0.0 0.0 0.0\nH 0.5 0.5 0.0\nH\t-0.5 0.5 0.0\n")
    s, mol = M.read_input(str(p))
    assert mol.natoms == 3 and list(mol.Z) == [8, 1, 1]
    assert np.allclose(mol.xyz[1], [0.5 * M.ANGSTROM_TO_BOHR, 0.5 * M.ANGSTROM_TO_BOHR, 0.0])
    assert (s.radial_points, s.lebedev_order, s.lmax) == (10, 4, 5)
    assert mol.nbf == 7


def test_nuclear_repulsion_h2():
    mol = M.Molecule([1, 1], [[0, 0, 0], [0, 0, 1.4]], "sto3g")
    assert abs(mol.nuclear_repulsion() - 1.0 / 1.4) < 1e-15


def test_synthetic_contraction_workload_is_seeded():
    a = M.synthetic_contraction(npts=1000, nbf=16, nocc=4)
    b = M.synthetic_contraction(npts=1000, nbf=16, nocc=4)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    pts, w, lmn, alpha, centres, P = a
    assert pts.min() >= 0 and pts.max() <= 20 and w.min() >= 1e-4 and w.max() <= 1.0
    assert alpha.min() >= 0.1 and alpha.max() <= 50 and np.allclose(P, P.T)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    r = bench.max_over_ranks([1.0 + rank, 10.0 - rank, 0.5 * rank])
    ref = bench.run_reference(None, rank) if rank != 0 else "rank0"
    out.put((rank, r, ref))
    dist.barrier()
    dist.destroy_process_group()


def test_bench_rank_reduction_two_gloo_ranks():
    """Replica timing takes the maximum over ranks; only rank 0 runs the CPU
    reference arm (the other ranks return without work)."""
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict()
    for _ in range(2):
        rank, r, ref = q.get(timeout=120)
        res[rank] = (r, ref)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank in (0, 1):
        assert res[rank][0] == [2.0, 10.0, 0.5]
    assert res[1][1] is None
