"""Device SCF driver (dftg_scf_*) against the host-driven SCF of the same
builds (grid.DFT: numpy eigen-solves, GPU Fock builds) and against the
oracle's reference SCF.

Tolerances (written per test):
  FP64, device vs host loop: same iteration count, per-iteration energies
      within 1e-9 Ha, final P within 1e-8;
  FP64, device vs the oracle's reference SCF: energies within 1e-8 Ha;
  mixed, device vs host mixed loop: 3e-8 Ha (both stop at |dE| <= 1e-8),
      iteration counts within three; device mixed vs host FP64: 1e-6 Ha (the
      mixed-precision energy bar).
"""
import numpy as np
import pytest

from dftcxx_gb300.molecule import Molecule, alkane, small_molecule

pytestmark = pytest.mark.gpu


def _host(mol, grid, precision, tol):
    from dftcxx_gb300.grid import DFT
    d = DFT(mol, *grid, precision=precision)
    E = d.scf(tol=tol)
    return d, E


def _device(mol, grid, precision, tol, **kw):
    from dftcxx_gb300.grid import DeviceSCF
    s = DeviceSCF(mol, *grid, precision=precision, tol=tol, **kw)
    E = s.run()
    return s, E


def test_device_scf_h2o_fp64_matches_host_loop(gpu_lib):
    Z, xyz = small_molecule("H2O")
    mol = Molecule(Z, xyz, "sto3g")
    grid = (32, 7, 8)
    d, Eh = _host(mol, grid, "fp64", 1e-8)
    s, Ed = _device(mol, grid, "fp64", 1e-8)
    assert abs(s.et - Ed) == 0.0
    hist = s.history()
    assert len(hist) == len(d.history), (len(hist), len(d.history))
    for row, h in zip(hist, d.history):
        assert abs(row[0] - h["E"]) <= 1e-9, (row[0], h["E"])
        assert abs(row[3] - h["Exc"]) <= 1e-9
    assert abs(Ed - Eh) <= 1e-9
    assert np.abs(s.P - d.P).max() <= 1e-8
    diag = s.diagnostics()
    assert diag["mode"] == 1, diag          # the whole loop ran as one conditional graph
    assert diag["orth"] <= 1e-12 and diag["cross"] <= 1e-10, diag
    X = s.matrix("X")
    S, _, _ = s.molgrid.one_electron()
    assert np.abs(X.T @ S @ X - np.eye(mol.nbf)).max() <= 1e-12
    eps = s.orbital_energies()
    F = s.matrix("H") + 2.0 * s.matrix("J") + s.matrix("XC")
    lam = np.linalg.eigvalsh(X.T @ F @ X)
    assert np.abs(np.sort(eps)[:mol.nelec // 2] - lam[:mol.nelec // 2]).max() <= 1e-3   # F moved after the last solve
    s.close()


def test_device_scf_h2o_fp64_matches_oracle_scf(gpu_lib):
    from oracle.oracle import OracleGrid, scf as oracle_scf
    Z, xyz = small_molecule("H2O")
    mol = Molecule(Z, xyz, "sto3g")
    grid = (24, 6, 6)
    hist, _ = oracle_scf(OracleGrid(mol, *grid), tol=1e-8)
    s, Ed = _device(mol, grid, "fp64", 1e-8)
    dh = s.history()
    assert len(dh) == len(hist)
    for row, h in zip(dh, hist):
        assert abs(row[0] - h["E"]) <= 1e-8, (row[0], h["E"])
    assert np.abs(s.P - hist[-1]["P"]).max() <= 1e-7
    s.close()


def test_device_scf_ethane_mixed(gpu_lib):
    Z, xyz = alkane(2)
    mol = Molecule(Z, xyz, "p631")
    grid = (50, 10, 8)
    _, Eh64 = _host(mol, grid, "fp64", 1e-8)
    dm, Ehm = _host(mol, grid, "mixed", 1e-8)
    s, Ed = _device(mol, grid, "mixed", 1e-8)
    # both loops stop at |dE| <= 1e-8 with different eigen-solvers, so each
    # final energy sits within a few 1e-8 of the common fixed point
    assert abs(Ed - Ehm) <= 3e-8, (Ed, Ehm)
    assert abs(Ed - Eh64) <= 1e-6, (Ed, Eh64)
    # the two loops cross the stopping threshold within a few iterations of each other
    assert abs(s.iterations - len(dm.history)) <= 3
    s.close()


def test_device_scf_step_matches_run(gpu_lib):
    from dftcxx_gb300.grid import DeviceSCF
    Z, xyz = small_molecule("NH3")
    mol = Molecule(Z, xyz, "p631")
    grid = (24, 7, 6)
    a = DeviceSCF(mol, *grid, precision="mixed", tol=1e-9, max_iter=12)
    Ea = a.run()
    ha = a.history()
    b = DeviceSCF(mol, *grid, precision="mixed", tol=1e-9, max_iter=12)
    es = []
    for _ in range(40):
        e, conv = b.step()
        es.append(e)
        if conv:
            break
    assert len(es) == len(ha)
    assert np.abs(np.array(es) - ha[:, 0]).max() == 0.0   # same graphs, same arithmetic
    assert es[-1] == Ea
    a.close()
    b.close()


def test_forces_after_device_scf(gpu_lib):
    """The SCF leaves a complete build of its final P: the backward pass runs
    on it (grid forces at the converged density)."""
    Z, xyz = small_molecule("CO")
    mol = Molecule(Z, xyz, "sto3g")
    s, _ = _device(mol, (24, 8, 6), "fp64", 1e-8)
    dP, dR = s.molgrid.backward()
    g2 = s.molgrid
    out = g2.fock_build(s.P)
    dP2, dR2 = g2.backward()
    assert np.abs(dR - dR2).max() <= 1e-12 * max(1.0, np.abs(dR).max())
    assert np.abs(dR.sum(axis=0)).max() <= 1e-8
    assert np.isfinite(out["Exc"])
    s.close()
