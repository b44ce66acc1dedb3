"""Persistent batch launches (DFTG_BATCH_PERSISTENT): every step of the mixed
build runs as one launch over all molecules of the batch, its CTAs taking
(molecule, block) work items from a device queue.

Checks:
  * the batch is bit-identical to each molecule's single build (J, XC, E_xc,
    N, E_J) eager, captured and replayed, before and after the batch autotuner
    (single builds with the same launch shapes), and the persistent form is the
    one that ran;
  * the graph-of-branches form (DFTG_BATCH_GRAPH) gives the same numbers;
  * the bounded wait of the fused atom-sum + point launch gives up on a flag
    that nothing sets: the self-test returns DFTG_ERR_TIMEOUT within a few
    limits, and the next batch is correct again."""
import time

import numpy as np
import pytest

from dftcxx_gb300.molecule import Molecule, small_molecule

pytestmark = pytest.mark.gpu

SPECS = [("H2", "sto3g"), ("LiH", "p631"), ("H2O", "sto3g"), ("NH3", "p631"), ("CH4", "sto3g"),
         ("N2", "p631"), ("CO", "sto3g"), ("C2H6", "p631"), ("C6H6", "p631"), ("C6H6", "sto3g")]


def _density(mol, seed):
    rng = np.random.default_rng(seed)
    C = rng.normal(0, 0.2, size=(mol.nbf, max(1, mol.nelec // 2)))
    return C @ C.T


@pytest.fixture(scope="module")
def batch_case(gpu_lib):
    import torch
    from dftcxx_gb300.grid import MolecularGrid
    rng = np.random.default_rng(11)
    grids, Ps = [], []
    for i, (name, basis) in enumerate(SPECS):
        Z, xyz = small_molecule(name)
        xyz = np.asarray(xyz, dtype=float) + rng.normal(0.0, 0.03, size=(len(Z), 3))
        mol = Molecule(Z, xyz, basis)
        grids.append(MolecularGrid(mol, 30, 8, 6, precision="mixed"))
        Ps.append(_density(mol, 40 + i))
    dev = torch.device("cuda")
    Pd = [torch.from_numpy(np.asfortranarray(P).ravel(order="F").copy()).to(dev) for P in Ps]
    yield grids, Ps, Pd
    for g in grids:
        g.close()


def _outputs(Ps):
    import torch
    dev = torch.device("cuda")
    Jd = [torch.zeros(P.size, dtype=torch.float64, device=dev) for P in Ps]
    Xd = [torch.zeros_like(j) for j in Jd]
    Sd = [torch.zeros(3, dtype=torch.float64, device=dev) for _ in Ps]
    return Jd, Xd, Sd


def _singles(grids, Ps):
    return [g.fock_build(P) for g, P in zip(grids, Ps)]


def _check(ref, Ps, Jd, Xd, Sd):
    for r, P, j, x, sc in zip(ref, Ps, Jd, Xd, Sd):
        n = P.shape[0]
        J1 = j.cpu().numpy().reshape(n, n, order="F")
        X1 = x.cpu().numpy().reshape(n, n, order="F")
        s = sc.cpu().numpy()
        assert np.array_equal(J1, r["J"]) and np.array_equal(X1, r["XC"])
        assert s[0] == r["Exc"] and s[2] == r["EJ"]


def test_persistent_batch_is_bit_identical_to_single_builds(batch_case):
    import torch
    from dftcxx_gb300.grid import Batch
    grids, Ps, Pd = batch_case
    ref = _singles(grids, Ps)
    Jd, Xd, Sd = _outputs(Ps)
    stream = torch.cuda.Stream()
    b = Batch(grids)
    for _ in range(3):                      # eager, captured, replayed
        with torch.cuda.stream(stream):
            for t in Jd + Xd + Sd:
                t.zero_()
        b.build(Pd, Jd, Xd, Sd, stream=stream.cuda_stream)
        b.status()
        assert b.persistent_active()
        _check(ref, Ps, Jd, Xd, Sd)
    # the autotuner changes the contexts' launch shapes: single builds with the
    # chosen shapes are again bit-identical to the batch
    b.autotune(reps=2)
    for _ in range(2):
        b.build(Pd, Jd, Xd, Sd, stream=stream.cuda_stream)
    b.status()
    _check(_singles(grids, Ps), Ps, Jd, Xd, Sd)
    # the graph of branches gives the same numbers
    b.set_mode("graph")
    for t in Jd + Xd + Sd:
        t.zero_()
    torch.cuda.synchronize()
    for _ in range(2):
        b.build(Pd, Jd, Xd, Sd, stream=stream.cuda_stream)
    b.status()
    assert not b.persistent_active()
    _check(_singles(grids, Ps), Ps, Jd, Xd, Sd)
    b.close()


def test_persistent_batch_wait_timeout_is_reported(batch_case):
    import torch
    from dftcxx_gb300 import _lib
    from dftcxx_gb300.grid import Batch
    grids, Ps, Pd = batch_case
    Jd, Xd, Sd = _outputs(Ps)
    stream = torch.cuda.Stream()
    b = Batch(grids)
    b.build(Pd, Jd, Xd, Sd, stream=stream.cuda_stream)
    b.status()
    t0 = time.perf_counter()
    rc = b.selftest_wait(20.0)
    dt = time.perf_counter() - t0
    assert rc == _lib.DFTG_ERR_TIMEOUT
    assert b"bounded wait" in _lib.load().dftg_last_error()
    assert dt < 5.0
    # the contexts and the batch stay usable: the next batch is correct
    for _ in range(2):
        b.build(Pd, Jd, Xd, Sd, stream=stream.cuda_stream)
    b.status()
    _check(_singles(grids, Ps), Ps, Jd, Xd, Sd)
    b.close()
