"""Backward pass of the grid energy (dftg_backward) against central finite
differences of the FP64 forward build, through the C ABI.

E = E_xc + E_J (E_J = 2 tr(P J) of the build) at fixed P.
  dE/dP: directional derivative along a random symmetric direction, step 1e-5.
  dE/dR: central differences with h = 1e-4 bohr; at a displaced geometry the
         grid and the basis functions move with their atoms (new context).
Tolerances (written per test):
  FP64 backward:  |dE/dR - FD| <= 2e-7 Ha/bohr, dE/dP directional 1e-7 relative;
  mixed forward + backward vs FD of the FP64 forward: <= 1e-5 Ha/bohr;
  translation sum rule: |sum_atoms dE/dR| <= 1e-8 Ha/bohr (FP64).
"""
import numpy as np
import pytest

from dftcxx_gb300.molecule import Molecule, alkane, small_molecule

pytestmark = pytest.mark.gpu


def _density(mol, seed=0):
    rng = np.random.default_rng(seed)
    C = rng.normal(0, 0.3, size=(mol.nbf, max(1, mol.nelec // 2)))
    return C @ C.T


def _grid(mol, nrad, leb, lmax, precision):
    from dftcxx_gb300.grid import MolecularGrid
    return MolecularGrid(mol, nrad, leb, lmax, precision=precision)


def _energy(mol, P, nrad, leb, lmax, seeds=(1.0, 1.0)):
    g = _grid(mol, nrad, leb, lmax, "fp64")
    out = g.fock_build(P)
    g.close()
    return seeds[0] * out["Exc"] + seeds[1] * out["EJ"]


def _fd_forces(mol, P, nrad, leb, lmax, coords, h=1e-4):
    fd = {}
    for (a, d) in coords:
        dx = np.zeros((mol.natoms, 3))
        dx[a, d] = h
        ep = _energy(mol.displaced(dx), P, nrad, leb, lmax)
        em = _energy(mol.displaced(-dx), P, nrad, leb, lmax)
        fd[(a, d)] = (ep - em) / (2 * h)
    return fd


def _backward(mol, P, nrad, leb, lmax, precision, seeds=(1.0, 1.0)):
    g = _grid(mol, nrad, leb, lmax, precision)
    g.fock_build(P)
    dP, dR = g.backward(*seeds)
    return g, dP, dR


def test_backward_h2o_fp64_matches_finite_differences(gpu_lib):
    Z, xyz = small_molecule("H2O")
    mol = Molecule(Z, xyz, "sto3g")
    nrad, leb, lmax = 32, 7, 8
    P = _density(mol)
    g, dP, dR = _backward(mol, P, nrad, leb, lmax, "fp64")
    # dE/dP along a random symmetric direction
    rng = np.random.default_rng(7)
    D = rng.normal(size=P.shape)
    D = 0.5 * (D + D.T)
    eps = 1e-5
    ep = g.fock_build(P + eps * D)
    em = g.fock_build(P - eps * D)
    fd = ((ep["Exc"] + ep["EJ"]) - (em["Exc"] + em["EJ"])) / (2 * eps)
    an = float(np.sum(dP * D))
    assert abs(an - fd) <= 1e-7 * abs(fd), (an, fd)
    assert np.abs(dP - dP.T).max() <= 1e-12 * np.abs(dP).max()
    # every nuclear coordinate
    coords = [(a, d) for a in range(mol.natoms) for d in range(3)]
    fd = _fd_forces(mol, P, nrad, leb, lmax, coords)
    err = max(abs(dR[a, d] - fd[(a, d)]) for (a, d) in coords)
    assert err <= 2e-7, (err, dR, fd)
    assert np.abs(dR.sum(axis=0)).max() <= 1e-8


def test_backward_seeds_are_linear(gpu_lib):
    Z, xyz = small_molecule("NH3")
    mol = Molecule(Z, xyz, "p631")
    P = _density(mol, 3)
    g, dP11, dR11 = _backward(mol, P, 16, 8, 6, "fp64")
    dP10, dR10 = g.backward(1.0, 0.0)
    dP01, dR01 = g.backward(0.0, 1.0)
    dP23, dR23 = g.backward(2.0, -3.0)
    sc = np.abs(dP11).max()
    assert np.abs(dP10 + dP01 - dP11).max() <= 1e-12 * sc
    assert np.abs(2 * dP10 - 3 * dP01 - dP23).max() <= 1e-12 * sc
    sr = np.abs(dR10).max() + np.abs(dR01).max()
    assert np.abs(dR10 + dR01 - dR11).max() <= 1e-12 * sr
    assert np.abs(2 * dR10 - 3 * dR01 - dR23).max() <= 1e-12 * sr


@pytest.mark.parametrize("seeds", [(1.0, 0.0), (0.0, 1.0)])
def test_backward_energy_parts_match_finite_differences(gpu_lib, seeds):
    """E_xc and E_J separately (the Hartree adjoint is not the forward's
    transpose in general: this checks the transposed operators)."""
    Z, xyz = small_molecule("CO")
    mol = Molecule(Z, xyz, "sto3g")
    nrad, leb, lmax = 24, 8, 8
    P = _density(mol, 5)
    g, dP, dR = _backward(mol, P, nrad, leb, lmax, "fp64", seeds)
    coords = [(0, 0), (0, 2), (1, 2)]
    h = 1e-4
    for (a, d) in coords:
        dx = np.zeros((mol.natoms, 3))
        dx[a, d] = h
        ep = _energy(mol.displaced(dx), P, nrad, leb, lmax, seeds)
        em = _energy(mol.displaced(-dx), P, nrad, leb, lmax, seeds)
        fd = (ep - em) / (2 * h)
        assert abs(dR[a, d] - fd) <= 2e-7, (a, d, dR[a, d], fd)


def test_backward_ethane_mixed_within_force_bar(gpu_lib):
    """Staggered ethane / 6-31G / 50 x 194: mixed forward + backward against
    FD of the FP64 forward, |error| <= 1e-5 Ha/bohr; the FP64 backward on the
    same coordinates as a control."""
    Z, xyz = alkane(2)
    mol = Molecule(Z, xyz, "p631")
    nrad, leb, lmax = 50, 10, 8
    P = _density(mol, 11)
    coords = [(0, 0), (0, 2), (1, 1), (2, 0), (5, 2)]
    fd = _fd_forces(mol, P, nrad, leb, lmax, coords)
    _, _, dR64 = _backward(mol, P, nrad, leb, lmax, "fp64")
    _, _, dRm = _backward(mol, P, nrad, leb, lmax, "mixed")
    e64 = max(abs(dR64[a, d] - fd[(a, d)]) for (a, d) in coords)
    em = max(abs(dRm[a, d] - fd[(a, d)]) for (a, d) in coords)
    assert e64 <= 2e-7, e64
    assert em <= 1e-5, em


def test_backward_decane_mixed_and_fp64(gpu_lib):
    """Decane / 6-31G / 50 x 194 (32 atoms, 134 functions) at the core-Hamiltonian
    guess density: FP64 backward against central differences on two
    coordinates (2e-7 Ha/bohr), the mixed forward + backward against the FP64
    backward (1e-5 Ha/bohr, every coordinate) and the translation sum rule
    (FP64 1e-8, mixed 1e-6)."""
    from dftcxx_gb300.grid import DFT
    Z, xyz = alkane(10)
    mol = Molecule(Z, xyz, "p631")
    nrad, leb, lmax = 50, 10, 8
    P = DFT(mol, nrad, leb, lmax, precision="fp64").P.copy()
    g, dP64, dR64 = _backward(mol, P, nrad, leb, lmax, "fp64")
    assert np.abs(dR64.sum(axis=0)).max() <= 1e-8
    coords = [(8, 0), (3, 1)]
    fd = _fd_forces(mol, P, nrad, leb, lmax, coords)
    err = max(abs(dR64[a, d] - fd[(a, d)]) for (a, d) in coords)
    assert err <= 2e-7, (err, [(dR64[a, d], fd[(a, d)]) for (a, d) in coords])
    g.set_precision("mixed")
    g.fock_build(P)
    dPm, dRm = g.backward()
    assert np.abs(dRm - dR64).max() <= 1e-5, np.abs(dRm - dR64).max()
    assert np.abs(dRm.sum(axis=0)).max() <= 1e-6
    assert np.abs(dPm - dP64).max() <= 1e-6 * np.abs(dP64).max()
