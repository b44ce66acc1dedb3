"""Two-electron integrals on the device (dftg_eri_list, dftg_eri_coulomb;
McMurchie-Davidson) against the oracle's restatement of the reference's
Taketa-Huzinaga-O-ohata formula (integrals.cpp:185-466), and the analytic J
against the grid J of the same build.

Tolerances: integrals and J within 1e-12 (absolute, values O(1)).
J_ERI against the Becke-Poisson J / c measures the grid's discretisation error
(the reference's grid algorithm, not an implementation error): benzene 75 x 302
/ lmax 8, measured 4.9e-5 of max |J| and 4.6e-3 Ha in 2 tr(P J) -> bounds 1e-4
of max |J| and 1e-2 Ha; ethane: the E_J error shrinks at least 5-fold from
50 x 194 / lmax 8 to 120 x 302 / lmax 12 (measured 1.6e-3 -> 9e-5 Ha)."""
import ctypes

import numpy as np
import pytest

from dftcxx_gb300.molecule import Molecule, alkane, benzene, small_molecule

pytestmark = pytest.mark.gpu


def _gpu_list(g, nbf):
    from dftcxx_gb300 import _lib
    npair = nbf * (nbf + 1) // 2
    out = np.zeros(npair * (npair + 1) // 2)
    _lib.check(_lib.load().dftg_eri_list(g.handle, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), out.size))
    return out


def _d_molecule():
    """H2O with an s + d basis on O (exercises the d-function form)."""
    Z, xyz = small_molecule("H2O")
    mol = Molecule(Z, xyz, "sto3g")
    data = {1: [("S", [(3.4252509, 0.1543290), (0.6239137, 0.5353281), (0.1688554, 0.4446345)])],
            8: [("S", [(130.70932, 0.1543290), (23.808861, 0.5353281), (6.4436083, 0.4446345)]),
                ("P", [(5.0331513, 0.1559163), (1.1695961, 0.6076837)]),
                ("D", [(1.2, 1.0)]), ("D", [(0.35, 0.6), (2.1, 0.4)])]}
    mol._build_basis(data)
    return mol


@pytest.mark.parametrize("case", ["h2o_sto3g", "nh3_631g", "h2o_d"])
def test_eri_list_matches_oracle(gpu_lib, case):
    from dftcxx_gb300.grid import MolecularGrid
    from oracle.oracle import OracleGrid
    if case == "h2o_d":
        mol = _d_molecule()
    else:
        name, basis = {"h2o_sto3g": ("H2O", "sto3g"), "nh3_631g": ("NH3", "p631")}[case]
        mol = Molecule(*small_molecule(name), basis)
    g = MolecularGrid(mol, 8, 4, 4)
    got = _gpu_list(g, mol.nbf)
    ref = OracleGrid(mol, 8, 4, 4).eri_list()
    assert np.abs(got - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max()), np.abs(got - ref).max()
    g.close()


def test_eri_coulomb_matches_oracle(gpu_lib):
    from dftcxx_gb300.grid import MolecularGrid
    from oracle.oracle import OracleGrid
    mol = Molecule(*small_molecule("NH3"), "p631")
    rng = np.random.default_rng(2)
    C = rng.normal(0, 0.3, size=(mol.nbf, 5))
    P = C @ C.T
    g = MolecularGrid(mol, 8, 4, 4)
    J = g.eri_coulomb(P)
    Jr = OracleGrid(mol, 8, 4, 4).eri_coulomb(P)
    assert np.abs(J - Jr).max() <= 1e-12 * np.abs(Jr).max()
    assert np.abs(J - J.T).max() == 0.0
    g.close()


def _grid_vs_eri(mol, P, grid):
    from dftcxx_gb300.grid import MolecularGrid
    g = MolecularGrid(mol, *grid, precision="fp64")
    Je = g.eri_coulomb(P)
    g.set_density(P)
    c = g.correct_densities()
    Jg = g.calculate_hartree_potential()
    g.close()
    return np.abs(Jg / c - Je).max(), np.abs(Je).max(), abs(2.0 * np.sum(P * (Jg - Je)))


def test_eri_coulomb_matches_grid_coulomb_benzene(gpu_lib):
    """The analytic J against the Becke-Poisson J of the FP64 build at the
    converged density (benzene / 6-31G / 75 x 302 / lmax 8)."""
    from dftcxx_gb300.grid import DeviceSCF
    mol = Molecule(*benzene(), "p631")
    s = DeviceSCF(mol, 75, 11, 8, precision="fp64", tol=1e-6)
    s.run()
    P = s.P
    s.close()
    err, jmax, dE = _grid_vs_eri(mol, P, (75, 11, 8))
    assert err <= 1e-4 * jmax, (err, jmax)
    assert dE <= 1e-2, dE


def test_grid_coulomb_converges_to_eri_coulomb(gpu_lib):
    from dftcxx_gb300.grid import DeviceSCF
    mol = Molecule(*alkane(2), "p631")
    s = DeviceSCF(mol, 50, 10, 8, precision="fp64", tol=1e-6)
    s.run()
    P = s.P
    s.close()
    _, _, d_coarse = _grid_vs_eri(mol, P, (50, 10, 8))
    _, _, d_fine = _grid_vs_eri(mol, P, (120, 11, 12))
    assert d_fine <= d_coarse / 5, (d_coarse, d_fine)
