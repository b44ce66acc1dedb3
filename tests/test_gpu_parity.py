"""FP64 CUDA path vs the CPU oracle, through the C ABI (libdftg.so).

Tolerances: the plain FP64 GPU build must reproduce the oracle's J, XC, E_xc
and the per-point arrays to 1e-10 (absolute for matrix elements and energies,
relative for point arrays)."""
import numpy as np
import pytest

from dftcxx_gb300.molecule import Molecule, h2o, benzene, small_molecule

pytestmark = pytest.mark.gpu

TOL = 1e-10


def _pair(gpu_lib, oracle_mod, mol, nrad, leb, lmax, precision="fp64"):
    from dftcxx_gb300.grid import MolecularGrid
    g = MolecularGrid(mol, nrad, leb, lmax, precision=precision)
    o = oracle_mod.OracleGrid(mol, nrad, leb, lmax)
    return g, o


def _density(mol, seed=0):
    rng = np.random.default_rng(seed)
    C = rng.normal(0, 0.3, size=(mol.nbf, max(1, mol.nelec // 2)))
    return C @ C.T


@pytest.mark.parametrize("name,basis,nrad,leb,lmax", [
    ("H2O", "sto3g", 32, 7, 8),
    ("LiH", "p631", 20, 5, 6),
    ("NH3", "p631", 16, 8, 8),
])
def test_grid_and_amplitudes(gpu_lib, oracle_mod, name, basis, nrad, leb, lmax):
    Z, xyz = small_molecule(name)
    mol = Molecule(Z, xyz, basis)
    g, o = _pair(gpu_lib, oracle_mod, mol, nrad, leb, lmax)
    assert g.grid_size == o.npts
    np.testing.assert_allclose(g.get_positions(), o.positions(), rtol=0, atol=1e-12)
    # Becke weights lie in [0, 1]: compare absolutely (tiny weights come from
    # cancelling distance differences and carry 1e-16 absolute noise)
    wb_o = o.becke_weights()
    assert np.abs(g.get_becke_weights() - wb_o).max() < 1e-13
    # total weights: relative 1e-12, plus the Becke-weight noise times the
    # geometric weight of the radial shell (points with w_becke ~ 0)
    w_o = o.weights()
    nang = g.grid_size // (mol.natoms * nrad)
    geom = np.where(wb_o > 1e-3, w_o / np.maximum(wb_o, 1e-3), 0.0).reshape(-1, nang).max(axis=1)
    tol = 1e-12 * np.abs(w_o) + 1e-13 * np.repeat(geom, nang)
    assert np.all(np.abs(g.get_weights() - w_o) <= tol)
    A = g.get_amplitudes()                       # nbf x npts
    np.testing.assert_allclose(A.T, o.amplitudes(), rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("name,basis,nrad,leb,lmax", [
    ("H2O", "sto3g", 32, 7, 8),
    ("CH4", "p631", 20, 8, 6),
    ("CO", "sto3g", 24, 10, 10),
])
def test_fock_build_fp64_matches_oracle(gpu_lib, oracle_mod, name, basis, nrad, leb, lmax):
    Z, xyz = small_molecule(name)
    mol = Molecule(Z, xyz, basis)
    g, o = _pair(gpu_lib, oracle_mod, mol, nrad, leb, lmax)
    P = _density(mol)
    ref = o.fock_build(P)
    out = g.fock_build(P)
    assert abs(out["nelec"] - ref["nelec"]) < TOL
    rho_o = o.densities()
    assert np.abs(g.get_densities() - rho_o).max() <= 1e-12 * np.abs(rho_o).max()
    np.testing.assert_allclose(g.get_potential(), o.potential(), rtol=1e-11, atol=1e-12)
    assert np.abs(out["J"] - ref["J"]).max() < TOL
    assert np.abs(out["XC"] - ref["XC"]).max() < TOL
    assert abs(out["Exc"] - ref["Exc"]) < TOL


def test_reference_call_sequence(gpu_lib, oracle_mod):
    """set_density -> correct_densities -> hartree -> xc, as DFT::scf calls them."""
    Z, xyz = h2o()
    mol = Molecule(Z, xyz, "sto3g")
    g, o = _pair(gpu_lib, oracle_mod, mol, 20, 7, 8)
    P = _density(mol, 3)
    g.set_density(P)
    o.set_density(P)
    assert abs(g.calculate_density() - o.calculate_density()) < TOL
    assert abs(g.correct_densities() - o.correct_densities()) < 1e-12
    assert abs(g.calculate_density() - mol.nelec) < 1e-9
    J = g.calculate_hartree_potential()
    assert np.abs(J - o.hartree()).max() < TOL
    XC, exc = g.calculate_xc()
    XCo, exco = o.xc()
    assert np.abs(XC - XCo).max() < TOL
    assert abs(exc - exco) < TOL


def test_one_electron_matches_oracle(gpu_lib, oracle_mod):
    for name, basis in (("H2O", "sto3g"), ("CO", "p631"), ("NH3", "p631")):
        Z, xyz = small_molecule(name)
        mol = Molecule(Z, xyz, basis)
        g, o = _pair(gpu_lib, oracle_mod, mol, 8, 0, 0)
        S, T, V = g.one_electron()
        So, To, Vo = o.one_electron()
        assert np.abs(S - So).max() < 1e-12
        assert np.abs(T - To).max() < 1e-11
        assert np.abs(V - Vo).max() < 1e-10
        assert abs(g.nuclear_repulsion() - o.nuclear_repulsion()) < 1e-12


def test_scf_h2o_fp64_matches_oracle(gpu_lib, oracle_mod):
    """H2O / STO-3G / 32 x 110, SCF from the core guess to dE < 1e-8."""
    from dftcxx_gb300.grid import DFT
    Z, xyz = h2o()
    mol = Molecule(Z, xyz, "sto3g")
    d = DFT(mol, 32, 7, 8, precision="fp64")
    e = d.scf(tol=1e-8)
    og = oracle_mod.OracleGrid(mol, 32, 7, 8)
    hist, _ = oracle_mod.scf(og, tol=1e-8)
    assert len(d.history) == len(hist)
    for a, b in zip(d.history, hist):
        assert abs(a["E"] - b["E"]) < TOL
        assert abs(a["Exc"] - b["Exc"]) < TOL
    assert abs(e - hist[-1]["E"]) < TOL


def test_mixed_precision_error_small(gpu_lib, oracle_mod):
    Z, xyz = h2o()
    mol = Molecule(Z, xyz, "sto3g")
    from dftcxx_gb300.grid import MolecularGrid
    g64 = MolecularGrid(mol, 32, 7, 8, precision="fp64")
    gmx = MolecularGrid(mol, 32, 7, 8, precision="mixed")
    P = _density(mol, 5)
    a = g64.fock_build(P)
    b = gmx.fock_build(P)
    assert np.abs(a["J"] - b["J"]).max() < 1e-5
    assert np.abs(a["XC"] - b["XC"]).max() < 1e-5
    assert abs(a["Exc"] - b["Exc"]) < 1e-5


@pytest.mark.parametrize("name,basis,nrad,leb", [("H2O", "sto3g", 32, 7), ("C6H6", "p631", 20, 8)])
def test_mixed_density_tensor_core_accuracy(gpu_lib, name, basis, nrad, leb):
    """The mixed-path density (integer-slice BF16 products on the tensor cores)
    reproduces the FP64 density to ~1e-10 relative."""
    from dftcxx_gb300.grid import MolecularGrid
    Z, xyz = small_molecule(name)
    mol = Molecule(Z, xyz, basis)
    g64 = MolecularGrid(mol, nrad, leb, 6, precision="fp64")
    gmx = MolecularGrid(mol, nrad, leb, 6, precision="mixed")
    P = _density(mol, 7)
    g64.set_density(P)
    gmx.set_density(P)
    r64, rmx = g64.get_densities(), gmx.get_densities()
    # four 8-bit slices per operand: 2^-33 of the row and column scales per
    # element, summed over nbf products, plus the FP32 rounding of the low-order
    # pairs (worst case a few 1e-8 at the nuclei)
    d = np.abs(rmx - r64)
    tol = 1e-7 * np.abs(r64) + 1e-12 * np.abs(r64).max()
    bad = np.argmax(d - tol)
    assert np.all(d <= tol), (float(d[bad]), float(r64[bad]), float(d.max()), float((d / np.maximum(r64, 1e-300)).max()))
    a, b = g64.fock_build(P), gmx.fock_build(P)
    assert abs(a["Exc"] - b["Exc"]) < 2e-7
    assert abs(a["EJ"] - b["EJ"]) < 2e-9 * abs(a["EJ"])


@pytest.mark.parametrize("name,basis,nrad,leb", [("H2O", "sto3g", 32, 7), ("C6H6", "p631", 20, 8)])
def test_mixed_contraction_tensor_core_accuracy(gpu_lib, name, basis, nrad, leb):
    """XC and J from the tensor-core contraction alone (all other steps FP64):
    integer leading slices make the leading sums exact, so the error is the
    FP32 rounding of the amplitudes and point coefficients."""
    from dftcxx_gb300.grid import MolecularGrid
    Z, xyz = small_molecule(name)
    mol = Molecule(Z, xyz, basis)
    g64 = MolecularGrid(mol, nrad, leb, 6, precision="fp64")
    gtc = MolecularGrid(mol, nrad, leb, 6, precision="fp64")
    gtc.set_precision_mask(MolecularGrid.MIX_BITS["contract"])
    P = _density(mol, 11)
    a, b = g64.fock_build(P), gtc.fock_build(P)
    dJ, dXC = np.abs(a["J"] - b["J"]).max(), np.abs(a["XC"] - b["XC"]).max()
    e_j = abs(2.0 * np.sum(P * (a["J"] - b["J"])))
    assert dJ < 1e-7 * np.abs(a["J"]).max() and dXC < 1e-7 * np.abs(a["XC"]).max(), (dJ, dXC, e_j)
    assert e_j < 2e-8 * abs(a["EJ"]), (dJ, dXC, e_j)
    assert np.abs(b["J"] - b["J"].T).max() == 0.0 and np.abs(b["XC"] - b["XC"].T).max() == 0.0


@pytest.mark.parametrize("name,basis,nrad,leb", [("H2O", "sto3g", 32, 7), ("C6H6", "p631", 20, 8)])
def test_mixed_correction_factor_from_sgrid(gpu_lib, name, basis, nrad, leb):
    """The whole mixed build takes the density correction's total from
    2 tr(P S_grid), S_grid = Phi^T diag(w) Phi made at set-up
    (moleculargrid.cpp:132-146).  Its corrected density then integrates to
    sum Z exactly when that total equals sum_p w rho of the same density: the
    reported N over sum Z is the ratio of the staged sequence's per-atom total
    to the S_grid total."""
    from dftcxx_gb300.grid import MolecularGrid
    Z, xyz = small_molecule(name)
    mol = Molecule(Z, xyz, basis)
    g = MolecularGrid(mol, nrad, leb, 6, precision="mixed")
    P = _density(mol, 5)
    r = g.fock_build(P)
    g.set_density(P)
    total = g.calculate_density()            # sum_p w rho of the mixed density, per-atom sums
    assert abs(total / mol.nelec - 1.0) > 1e-6   # a density that needs the correction
    assert abs(r["nelec"] - mol.nelec) < 1e-8 * mol.nelec, (r["nelec"], mol.nelec, total)
    g.close()


def test_batched_builds_match_single_builds(gpu_lib):
    """Four molecules of different sizes and precisions built in one captured
    launch give the same J, XC and energies as their single builds."""
    import torch
    from dftcxx_gb300.grid import MolecularGrid, Batch
    specs = [("H2O", "sto3g", "mixed"), ("NH3", "p631", "fp64"), ("CH4", "p631", "mixed"), ("CO", "sto3g", "mixed")]
    grids, Ps = [], []
    for i, (name, basis, prec) in enumerate(specs):
        Z, xyz = small_molecule(name)
        mol = Molecule(Z, xyz, basis)
        grids.append(MolecularGrid(mol, 20, 8, 6, precision=prec))
        Ps.append(_density(mol, 20 + i))
    ref = []
    for g, P in zip(grids, Ps):
        r = g.fock_build(P)
        ref.append((r["J"], r["XC"], r["Exc"], r["EJ"]))
    dev = torch.device("cuda")
    Pd = [torch.from_numpy(np.asfortranarray(P).ravel(order="F").copy()).to(dev) for P in Ps]
    Jd = [torch.zeros(P.size, dtype=torch.float64, device=dev) for P in Ps]
    Xd = [torch.zeros_like(j) for j in Jd]
    Sd = [torch.zeros(3, dtype=torch.float64, device=dev) for _ in Ps]
    b = Batch(grids)
    for _ in range(3):                      # eager, captured, replayed
        for j in Jd + Xd:
            j.zero_()
        # the batch runs on the contexts' non-blocking streams, which do not
        # wait for torch's stream: the fills and the copies of P finish first
        torch.cuda.synchronize()
        b.build(Pd, Jd, Xd, Sd)
        torch.cuda.synchronize()
        for (J0, X0, e0, ej0), P, j, x, sc in zip(ref, Ps, Jd, Xd, Sd):
            n = P.shape[0]
            J1 = j.cpu().numpy().reshape(n, n, order="F")
            X1 = x.cpu().numpy().reshape(n, n, order="F")
            s = sc.cpu().numpy()
            assert np.array_equal(J1, J0) and np.array_equal(X1, X0)
            assert s[0] == e0 and s[2] == ej0
    # after the batch autotuner the batch still equals single builds of the
    # same launch shapes, and the contexts agree with their untuned results
    b.autotune(reps=2)
    for _ in range(3):
        b.build(Pd, Jd, Xd, Sd)
    torch.cuda.synchronize()
    for (J0, X0, e0, ej0), g, P, j, x in zip(ref, grids, Ps, Jd, Xd):
        n = P.shape[0]
        J1 = j.cpu().numpy().reshape(n, n, order="F")
        X1 = x.cpu().numpy().reshape(n, n, order="F")
        r = g.fock_build(P)
        assert np.array_equal(J1, r["J"]) and np.array_equal(X1, r["XC"])
        assert np.abs(J1 - J0).max() <= 1e-7 * np.abs(J0).max()
        assert np.abs(X1 - X0).max() <= 1e-7 * np.abs(X0).max()
    b.close()


def test_mixed_forward_decane_matches_fp64(gpu_lib):
    """32 atoms, 134 functions, 50 x 194: the mixed build (pair bins of the
    cross-atom potential, FP32 CUDA-core contraction beyond 128 functions)
    against the FP64 build at the core-Hamiltonian guess density:
    |dE_xc + dE_J| <= 1e-5 Ha, every potential value finite and within 1e-4."""
    from dftcxx_gb300.grid import DFT, MolecularGrid
    from dftcxx_gb300.molecule import alkane
    Z, xyz = alkane(10)
    mol = Molecule(Z, xyz, "p631")
    P = DFT(mol, 50, 10, 8, precision="fp64").P.copy()
    g = MolecularGrid(mol, 50, 10, 8, precision="fp64")
    r64 = g.fock_build(P)
    V64 = g.get_potential()
    g.set_precision("mixed")
    rm = g.fock_build(P)
    Vm = g.get_potential()
    assert np.all(np.isfinite(Vm))
    assert np.abs(Vm - V64).max() <= 1e-4
    assert abs((rm["Exc"] + rm["EJ"]) - (r64["Exc"] + r64["EJ"])) <= 1e-5


def test_autotune_keeps_results(gpu_lib):
    """The autotuner changes launch shapes only: builds before and after agree
    (split-K order changes the rounding: 1e-7 of max|J|, max|XC|), the chosen
    shape lies inside the allowed range and out-of-range shapes are refused."""
    from dftcxx_gb300 import _lib
    from dftcxx_gb300.grid import MolecularGrid
    from dftcxx_gb300.molecule import benzene
    Z, xyz = benzene()
    mol = Molecule(Z, xyz, "p631")
    g = MolecularGrid(mol, 40, 10, 8, precision="mixed")
    P = _density(mol, 2)
    r0 = g.fock_build(P)
    shape0 = g.launch_shape
    assert shape0[0] > 0 and shape0[1] > 0 and shape0[2] >= 2
    ms = g.autotune(reps=2)
    assert ms > 0.0
    shape1 = g.launch_shape
    assert 1 <= shape1[0] <= shape0[0] and 1 <= shape1[1] <= shape0[1] and 2 <= shape1[2] <= shape0[2]
    assert shape1[2] % 2 == 0
    r1 = g.fock_build(P)
    assert np.abs(r1["J"] - r0["J"]).max() <= 1e-7 * np.abs(r0["J"]).max()
    assert np.abs(r1["XC"] - r0["XC"]).max() <= 1e-7 * np.abs(r0["XC"]).max()
    assert abs(r1["Exc"] - r0["Exc"]) <= 1e-9 * abs(r0["Exc"])
    # an explicit shape, then the refusal of one beyond the setup maximum
    g.launch_shape = (max(1, shape0[0] // 2), max(1, shape0[1] // 2), shape1[2])
    r2 = g.fock_build(P)
    assert np.abs(r2["J"] - r0["J"]).max() <= 1e-7 * np.abs(r0["J"]).max()
    with pytest.raises(_lib.DftgError):
        g.launch_shape = (shape0[0] + 1, shape0[1], shape0[2])


def _synthetic_grid(npts, nbf, nocc, precision, seed=20261203):
    from dftcxx_gb300.grid import PointGrid
    from dftcxx_gb300.molecule import synthetic_contraction
    pts, w, lmn, alpha, centres, P = synthetic_contraction(npts=npts, nbf=nbf, nocc=nocc, seed=seed)
    g = PointGrid(pts, w, centres, np.arange(nbf), lmn, np.ones(nbf, np.int32), alpha, np.ones(nbf),
                  precision=precision)
    return g, (pts, w, lmn, alpha, centres, P)


@pytest.mark.parametrize("nbf", [1024, 1025])
def test_points_context_basis_limits(gpu_lib, oracle_mod, nbf):
    """The largest basis of the tiled tensor-core density and contraction (1024
    functions: eight row blocks, 36 contraction tiles, integer leading sums of
    the density up to 2^24) and the first one past it (1025: the FP32 CUDA-core
    kernels) on 8192 points: mixed rho, E_xc and XC within the tolerances of the
    smaller sets against the oracle."""
    g, (pts, w, lmn, alpha, centres, P) = _synthetic_grid(8192, nbf, nbf // 4, "mixed")
    e_o, rho_o, xc_o = oracle_mod.points_xc(pts, w, centres, np.arange(nbf), lmn, np.ones(nbf, np.int32), alpha,
                                            np.ones(nbf), P)
    rm = g.xc_build(P)
    assert np.abs(g.get_densities() - rho_o).max() <= 1e-6 * np.abs(rho_o).max()
    assert abs(rm["Exc"] - e_o) <= 1e-7 * abs(e_o)
    assert np.abs(rm["XC"] - xc_o).max() <= 1e-6 * np.abs(xc_o).max()
    g.close()


@pytest.mark.parametrize("nbf", [48, 133, 160, 200, 300, 512])
def test_points_context_matches_oracle(gpu_lib, oracle_mod, nbf):
    """Synthetic contraction workload (explicit points and function centres, no
    atoms) at a reduced size: the FP64 form reproduces the oracle's rho, E_xc
    and XC to 1e-10 (relative); the mixed form stays within 1e-6 of max|XC|,
    1e-6 of max rho and 1e-7 of |E_xc|.  Mixed density: tensor cores up to 80
    functions, register-tiled FP32 CUDA cores beyond (133 has padded P rows,
    200 ragged 128 x 64 tiles).  Mixed XC contraction: one tensor-core kernel
    up to 128 functions, 128 x 128 tensor-core tiles beyond (133: two row
    blocks, the second nearly empty; 300: six tiles, a ragged last block; 512:
    ten full tiles)."""
    g, (pts, w, lmn, alpha, centres, P) = _synthetic_grid(20_000, nbf, nbf // 4, "fp64")
    r = g.xc_build(P)
    rho = g.get_densities()
    e_o, rho_o, xc_o = oracle_mod.points_xc(pts, w, centres, np.arange(nbf), lmn, np.ones(nbf, np.int32), alpha,
                                            np.ones(nbf), P)
    np.testing.assert_allclose(rho, rho_o, rtol=1e-12, atol=1e-14 * np.abs(rho_o).max())
    assert abs(r["Exc"] - e_o) <= 1e-10 * abs(e_o)
    assert np.abs(r["XC"] - xc_o).max() <= 1e-10 * np.abs(xc_o).max()
    assert abs(r["nelec"] - float(w @ rho_o)) <= 1e-10 * abs(float(w @ rho_o))
    g.set_precision("mixed")
    rm = g.xc_build(P)
    assert np.abs(g.get_densities() - rho_o).max() <= 1e-6 * np.abs(rho_o).max()
    assert abs(rm["Exc"] - e_o) <= 1e-7 * abs(e_o)
    assert np.abs(rm["XC"] - xc_o).max() <= 1e-6 * np.abs(xc_o).max()
    from dftcxx_gb300 import _lib
    with pytest.raises(_lib.DftgError):
        g.fock_build(P)
