"""Oracle two-electron integrals (restatement of Integrator::repulsion,
integrals.cpp:185-466, and DFT::calculate_hartree_potential_te_int,
dft.cpp:452-477), pinned by
  * the H2 / STO-3G integrals at R = 1.4 bohr of Szabo and Ostlund, "Modern
    Quantum Chemistry" (1989), eq. 3.235: (11|11) 0.7746, (11|22) 0.5697,
    (21|11) 0.4441, (21|21) 0.2970 (four decimals);
  * the 8-fold permutational symmetry of (ij|kl);
  * an independent method: the Becke-Poisson grid J of the same oracle
    (divided by its density-correction factor) converges to J = sum P (ij|kl)
    as the grid is refined."""
import numpy as np
import pytest

from dftcxx_gb300.molecule import Molecule, small_molecule
from oracle.oracle import OracleGrid


def test_h2_sto3g_szabo_ostlund():
    mol = Molecule([1, 1], [[0, 0, 0], [0, 0, 1.4]], "sto3g")
    g = OracleGrid(mol, 8, 4, 4)
    ref = {(0, 0, 0, 0): 0.7746, (0, 0, 1, 1): 0.5697, (1, 0, 0, 0): 0.4441, (1, 0, 1, 0): 0.2970}
    for q, v in ref.items():
        assert abs(g.eri(*q) - v) < 6e-5, (q, g.eri(*q), v)


def test_eri_symmetry_and_list_order():
    Z, xyz = small_molecule("NH3")
    mol = Molecule(Z, xyz, "p631")
    g = OracleGrid(mol, 8, 4, 4)
    rng = np.random.default_rng(3)
    for _ in range(40):
        i, j, k, l = (int(x) for x in rng.integers(0, mol.nbf, 4))
        v = g.eri(i, j, k, l)
        for p in [(j, i, k, l), (i, j, l, k), (k, l, i, j), (l, k, j, i)]:
            assert abs(g.eri(*p) - v) <= 1e-14 * max(1.0, abs(v))
    lst = g.eri_list()
    def tidx(i, j, k, l):
        i, j = max(i, j), min(i, j)
        k, l = max(k, l), min(k, l)
        ij, kl = i * (i + 1) // 2 + j, k * (k + 1) // 2 + l
        ij, kl = max(ij, kl), min(ij, kl)
        return ij * (ij + 1) // 2 + kl
    for _ in range(40):
        q = tuple(int(x) for x in rng.integers(0, mol.nbf, 4))
        assert lst[tidx(*q)] == g.eri(*q) or abs(lst[tidx(*q)] - g.eri(*q)) <= 1e-14


def test_eri_coulomb_matches_grid_coulomb():
    Z, xyz = small_molecule("H2O")
    mol = Molecule(Z, xyz, "p631")
    rng = np.random.default_rng(0)
    C = rng.normal(0, 0.3, size=(mol.nbf, 5))
    P = C @ C.T
    Je = OracleGrid(mol, 8, 4, 4).eri_coulomb(P)
    assert np.abs(Je - Je.T).max() == 0.0
    errs = []
    for grid in [(32, 7, 6), (64, 10, 8)]:
        g = OracleGrid(mol, *grid)
        g.set_density(P)
        c = g.correct_densities()
        errs.append(np.abs(g.hartree() / c - Je).max())
    assert errs[1] < errs[0] / 5 and errs[1] < 3e-4, errs
