"""The oracle against the reference PROGRAM itself (CPU, no GPU needed).

The fixtures ref_h2o_sto3g_32x110.npz and ref_benzene_p631_75x302.npz hold what
the reference's own grid, Hartree, XC, energy and SCF code computes: its
unmodified translation units compiled against the Eigen/Boost API subset of
oracle/shim and run by tests/golden/make_goldens.py.  Here the C restatement
(oracle/dftg_oracle.c) must reproduce them on the same inputs.

Tolerances (absolute unless stated):
  SCF energies per iteration           1e-10 Ha, same iteration count
  J, XC, E_xc, E_J, N, S/T/V           1e-12
  weights, Becke weights               1e-12 relative
  rho                                  1e-12 relative to max rho
  V_H (per point)                      1e-11
  rho_lm                               1e-11 relative to max |rho_lm|
  U_lm                                 1e-10 relative to max |U_lm| (both sides solve
                                       the Poisson systems by their own pivoted LU)
When oracle/_ref has been built here (the reference sources are present), the
reference program is also run live on a small case and compared directly.
"""
import os

import numpy as np
import pytest

from dftcxx_gb300.molecule import Molecule, benzene, h2o, parse_basis_dat

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    return dict(np.load(os.path.join(GOLD, name)))


def _relmax(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max())


def test_oracle_scf_matches_reference_program_h2o(oracle_mod):
    ref = _load("ref_h2o_sto3g_32x110.npz")
    Z, xyz = h2o()
    g = oracle_mod.OracleGrid(Molecule(Z, xyz, "sto3g"), 32, 7, 8)
    hist, _ = oracle_mod.scf(g, tol=1e-10)
    E = np.array([h["E"] for h in hist])
    assert len(E) == len(ref["history"])
    assert np.abs(E - ref["history"][:, 0]).max() <= 1e-10
    assert np.abs(np.array([h["Exc"] for h in hist]) - ref["history"][:, 3]).max() <= 1e-10
    assert np.abs(hist[-1]["P"] - ref["P"]).max() <= 1e-10


def test_oracle_build_matches_reference_program_h2o(oracle_mod):
    ref = _load("ref_h2o_sto3g_32x110.npz")
    Z, xyz = h2o()
    mol = Molecule(Z, xyz, "sto3g")
    g = oracle_mod.OracleGrid(mol, 32, 7, 8)
    P = ref["P"]
    np.testing.assert_allclose(g.weights(), ref["w"], rtol=1e-12, atol=0)
    np.testing.assert_allclose(g.becke_weights(), ref["becke"], rtol=1e-12, atol=1e-300)
    g.set_density(P)
    n0 = g.calculate_density()
    g.correct_densities()
    J = g.hartree()
    XC, exc = g.xc()
    S, T, V = g.one_electron()
    exc_r, ej_r, eone_r, enuc_r, etot_r, n0_r, n1_r = ref["scalars"]
    assert abs(n0 - n0_r) <= 1e-12
    assert np.abs(J - ref["J"]).max() <= 1e-12
    assert np.abs(XC - ref["XC"]).max() <= 1e-12
    assert abs(exc - exc_r) <= 1e-12
    assert abs(2 * np.trace(P @ J) - ej_r) <= 1e-12
    assert abs(g.nuclear_repulsion() - enuc_r) <= 1e-12
    for a, b in ((S, ref["S"]), (T, ref["T"]), (V, ref["Vnuc"])):
        assert np.abs(a - b).max() <= 1e-12
    assert _relmax(g.densities(), ref["rho"]) <= 1e-12
    assert np.abs(g.potential() - ref["V"]).max() <= 1e-11
    assert _relmax(g.rho_lm(), ref["rho_lm"]) <= 1e-11
    assert _relmax(g.U_lm(), ref["U_lm"]) <= 1e-10


def test_oracle_build_matches_reference_program_benzene_75x302(oracle_mod):
    """The headline configuration: benzene / 6-31G / 75 x 302 (the 302-point
    rule added to the reference's table), lmax 8, at the density of the
    reference's own SCF."""
    ref = _load("ref_benzene_p631_75x302.npz")
    Z, xyz = benzene()
    g = oracle_mod.OracleGrid(Molecule(Z, xyz, "p631"), 75, 11, 8)
    P = ref["P"]
    idx = ref["idx"]
    w = g.weights()
    np.testing.assert_allclose(w[idx], ref["w"], rtol=1e-12, atol=0)
    np.testing.assert_allclose(g.becke_weights()[idx], ref["becke"], rtol=1e-12, atol=1e-300)
    g.set_density(P)
    n0 = g.calculate_density()
    g.correct_densities()
    J = g.hartree()
    XC, exc = g.xc()
    exc_r, ej_r, eone_r, enuc_r, etot_r, n0_r, n1_r = ref["scalars"]
    assert abs(n0 - n0_r) <= 1e-11
    assert np.abs(J - ref["J"]).max() <= 1e-12
    assert np.abs(XC - ref["XC"]).max() <= 1e-12
    assert abs(exc - exc_r) <= 1e-11
    assert abs(2 * np.trace(P @ J) - ej_r) <= 1e-11
    rho, V = g.densities(), g.potential()
    assert np.abs(rho[idx] - ref["rho"]).max() <= 1e-12 * np.abs(ref["rho"]).max()
    assert np.abs(V[idx] - ref["V"]).max() <= 1e-11
    sums = np.array([w.sum(), (w * rho).sum(), (w * V).sum(), (w * rho * V).sum(), g.becke_weights().sum()])
    np.testing.assert_allclose(sums, ref["sums"], rtol=1e-12)


def test_reference_basis_file_roundtrip():
    """The .dat files the reference program is given (written from the JSON
    basis data) parse to the numbers of the reference's own files."""
    import hashlib
    import json
    from oracle import refprog
    gold = json.load(open(os.path.join(GOLD, "ref_basis.json")))
    for name, rec in gold.items():
        data = parse_basis_dat(refprog.basis_dat(name))
        flat = np.array([v for z in sorted(data) for _, prims in data[z] for p in prims for v in p])
        assert hashlib.sha256(flat.tobytes()).hexdigest() == rec["sha256"], name


def test_reference_program_live_if_built(oracle_mod):
    """Where oracle/_ref holds the reference program (built from its sources
    here), run it on H2O / STO-3G / 16 x 50 / lmax 6 at a seeded P and compare
    with the oracle."""
    from oracle import refprog
    if not refprog.available(4):
        pytest.skip("oracle/_ref/ref_dump not built (needs the reference sources)")
    Z, xyz = h2o()
    mol = Molecule(Z, xyz, "sto3g", "water")
    rng = np.random.default_rng(5)
    C = rng.normal(0, 0.3, size=(mol.nbf, mol.nelec // 2))
    P = C @ C.T
    r = refprog.fock_build(mol, 16, 4, 6, P, amp=True)
    g = oracle_mod.OracleGrid(mol, 16, 4, 6)
    o = g.fock_build(P)
    assert np.abs(o["J"] - r["J"]).max() <= 1e-12
    assert np.abs(o["XC"] - r["XC"]).max() <= 1e-12
    assert abs(o["Exc"] - r["scalars"][0]) <= 1e-12
    assert _relmax(g.densities(), r["rho"]) <= 1e-12
    assert _relmax(g.amplitudes(), r["amplitudes"].T) <= 1e-14
