"""The CUDA build against the reference PROGRAM's own outputs (GPU).

Fixtures (tests/golden/ref_*.npz) are what the reference's unmodified grid,
Hartree, XC, energy and SCF code computed, run by tests/golden/make_goldens.py;
tests/test_reference_pin.py pins the C oracle to the same fixtures on the CPU.

Tolerances:
  FP64 CUDA build vs reference, at the reference's P:
    J, XC, E_xc, E_J                    1e-10 absolute
    rho                                 1e-12 relative to max rho
    V_H per point                       1e-11 relative, plus 1e-12 absolute
    Becke weights                       1e-12 absolute (tiny weights come from
                                        cancelling distance differences, products of
                                        up to 11 cut-off factors here; the device
                                        rounds them with fused multiply-adds)
    weights                             1e-12 relative, plus 1e-12 of the point's
                                        geometric weight w / w_becke (the same
                                        Becke-weight rounding, scaled)
    S, T, V (one-electron), E_nuc       1e-10 absolute
  mixed CUDA build vs reference, same P (benzene / 6-31G / 75 x 302):
    |dE_tot| = |dE_J + dE_xc|           1e-6 Ha (the metric's bar)
    max|dJ|, max|dXC|                   1e-6
  FP64 device SCF vs the reference's SCF (H2O / STO-3G / 32 x 110):
    converged energy                    1e-10 Ha, same iteration count
    energies per iteration              1e-9 Ha (eigen-solver rounding carried
                                        through the damped iterations)
    final P                             1e-7
"""
import os

import numpy as np
import pytest

from dftcxx_gb300.molecule import Molecule, benzene, h2o

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    return dict(np.load(os.path.join(GOLD, name)))


@pytest.fixture(scope="module")
def benzene_ref():
    return _load("ref_benzene_p631_75x302.npz")


def _check_weights(w, wb, ref):
    assert np.abs(wb - ref["becke"]).max() <= 1e-12
    geom = np.where(wb > 0, w / np.where(wb > 0, wb, 1.0), 0.0)
    geom = np.maximum(geom, np.where(ref["becke"] > 0, ref["w"] / np.where(ref["becke"] > 0, ref["becke"], 1.0), 0.0))
    assert np.all(np.abs(w - ref["w"]) <= 1e-12 * np.abs(ref["w"]) + 1e-12 * geom)


def _check_fp64(g, ref, P, idx=None):
    sel = (lambda a: a) if idx is None else (lambda a: a[idx])
    _check_weights(sel(g.get_weights()), sel(g.get_becke_weights()), ref)
    r = g.fock_build(P)
    exc_r, ej_r, eone_r, enuc_r = ref["scalars"][:4]
    assert np.abs(r["J"] - ref["J"]).max() <= 1e-10
    assert np.abs(r["XC"] - ref["XC"]).max() <= 1e-10
    assert abs(r["Exc"] - exc_r) <= 1e-10
    assert abs(r["EJ"] - ej_r) <= 1e-10
    rho = sel(g.get_densities())
    assert np.abs(rho - ref["rho"]).max() <= 1e-12 * np.abs(ref["rho"]).max()
    np.testing.assert_allclose(sel(g.get_potential()), ref["V"], rtol=1e-11, atol=1e-12)
    S, T, V = g.one_electron()
    for a, b in ((S, ref["S"]), (T, ref["T"]), (V, ref["Vnuc"])):
        assert np.abs(a - b).max() <= 1e-10
    assert abs(g.nuclear_repulsion() - enuc_r) <= 1e-10
    return r


def test_fp64_build_matches_reference_program_h2o(gpu_lib):
    from dftcxx_gb300.grid import MolecularGrid
    ref = _load("ref_h2o_sto3g_32x110.npz")
    Z, xyz = h2o()
    g = MolecularGrid(Molecule(Z, xyz, "sto3g"), 32, 7, 8, precision="fp64")
    _check_fp64(g, ref, ref["P"])
    g.close()


def test_fp64_build_matches_reference_program_benzene_75x302(gpu_lib, benzene_ref):
    """The headline configuration in FP64: benzene / 6-31G / 75 x 302 / lmax 8
    at the density of the reference's own SCF."""
    from dftcxx_gb300.grid import MolecularGrid
    ref = benzene_ref
    Z, xyz = benzene()
    g = MolecularGrid(Molecule(Z, xyz, "p631"), 75, 11, 8, precision="fp64")
    assert g.grid_size == 271800
    _check_fp64(g, ref, ref["P"], ref["idx"])
    w, rho, V = g.get_weights(), g.get_densities(), g.get_potential()
    sums = np.array([w.sum(), (w * rho).sum(), (w * V).sum(), (w * rho * V).sum(), g.get_becke_weights().sum()])
    np.testing.assert_allclose(sums, ref["sums"], rtol=1e-11)
    g.close()


def test_mixed_build_matches_reference_program_benzene_75x302(gpu_lib, benzene_ref):
    """The headline configuration in mixed precision against the reference:
    |dE_tot| <= 1e-6 Ha, max|dJ| and max|dXC| <= 1e-6 at the same P."""
    from dftcxx_gb300.grid import MolecularGrid
    ref = benzene_ref
    Z, xyz = benzene()
    g = MolecularGrid(Molecule(Z, xyz, "p631"), 75, 11, 8, precision="mixed")
    P = ref["P"]
    r = g.fock_build(P)
    exc_r, ej_r = ref["scalars"][:2]
    dE = (r["EJ"] - ej_r) + (r["Exc"] - exc_r)
    dJ = np.abs(r["J"] - ref["J"]).max()
    dXC = np.abs(r["XC"] - ref["XC"]).max()
    assert abs(dE) <= 1e-6, dE
    assert dJ <= 1e-6, dJ
    assert dXC <= 1e-6, dXC
    # the energy through the J matrix itself (as the reference forms it, 2 tr(P J))
    assert abs(2 * np.trace(P @ r["J"]) - ej_r) <= 2e-6
    g.close()


def test_device_scf_matches_reference_program_scf_h2o(gpu_lib):
    from dftcxx_gb300.grid import DeviceSCF
    ref = _load("ref_h2o_sto3g_32x110.npz")
    Z, xyz = h2o()
    s = DeviceSCF(Molecule(Z, xyz, "sto3g"), 32, 7, 8, precision="fp64", tol=1e-10)
    s.run()
    hist = np.asarray(s.history())
    assert len(hist) == len(ref["history"]), (len(hist), len(ref["history"]))
    assert abs(hist[-1, 0] - ref["history"][-1, 0]) <= 1e-10
    assert np.abs(hist[:, 0] - ref["history"][:, 0]).max() <= 1e-9
    assert np.abs(s.P - ref["P"]).max() <= 1e-7
    s.close()
