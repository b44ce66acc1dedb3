"""dftg_contract_noalloc: the XC / J contraction for callers that may not
allocate device memory while they serve (their framework owns all GPU memory,
or they run under a fixed device-memory budget).

The entry point is called through the C ABI on caller-owned device buffers,
twice in a row (the second call reuses the static scratch the first one left
behind).  Results are checked to 1e-10 (relative to the largest element
where the matrices are large):
  * H2O / STO-3G (7 functions, one diagonal 64 x 64 tile) against the
    context's own entry points (dftg_calculate_hartree_potential and
    dftg_calculate_xc);
  * 130 functions on a point-set context (three row blocks: off-diagonal tiles
    and their mirrored writes, a ragged last block), amplitude rows padded to
    a stride ld > npts, against the context's FP64 XC and against FP64 numpy;
  * 1024 functions, the limit, where one chunk of split-K partial sums fills
    the whole scratch array, against FP64 numpy.
This file is collected last so that a stop-at-first-failure run has already
run every other test."""
import ctypes

import numpy as np
import pytest

from dftcxx_gb300.molecule import Molecule, h2o

pytestmark = pytest.mark.gpu


def test_contract_noalloc_matches_context_entry_points(gpu_lib, oracle_mod):
    import torch
    from dftcxx_gb300 import _lib
    from dftcxx_gb300.grid import MolecularGrid

    Z, xyz = h2o()
    mol = Molecule(Z, xyz, "sto3g")
    g = MolecularGrid(mol, 32, 7, 8, precision="fp64")
    rng = np.random.default_rng(11)
    C = rng.normal(0, 0.3, size=(mol.nbf, mol.nelec // 2))
    P = C @ C.T
    g.set_density(P)
    g.correct_densities()
    J_ref = g.calculate_hartree_potential()
    XC_ref, _ = g.calculate_xc()

    # point coefficients of the two contractions, from the context's arrays
    w, V, rho = g.get_weights(), g.get_potential(), g.get_densities()
    L = oracle_mod.lib()
    v = np.empty_like(rho)
    e_, v_ = ctypes.c_double(), ctypes.c_double()
    for i, r in enumerate(rho):
        L.orc_lda_point(float(r), ctypes.byref(e_), ctypes.byref(v_))
        v[i] = v_.value
    cxc = w * v
    cj = 0.5 * (w * V)
    phi = np.ascontiguousarray(g.get_amplitudes())          # nbf x npts, row stride npts

    dev = torch.device("cuda:0")
    phi_d = torch.from_numpy(phi).to(dev)
    cxc_d = torch.from_numpy(cxc).to(dev)
    cj_d = torch.from_numpy(cj).to(dev)
    lib = _lib.load()
    nbf, npts = phi.shape
    for call in range(2):
        XC_d = torch.full((nbf * nbf,), float("nan"), dtype=torch.float64, device=dev)
        J_d = torch.full((nbf * nbf,), float("nan"), dtype=torch.float64, device=dev)
        rc = lib.dftg_contract_noalloc(ctypes.c_void_p(phi_d.data_ptr()), npts, npts, nbf,
                                       ctypes.c_void_p(cxc_d.data_ptr()), ctypes.c_void_p(cj_d.data_ptr()),
                                       ctypes.c_void_p(XC_d.data_ptr()), ctypes.c_void_p(J_d.data_ptr()), None)
        _lib.check(rc)
        torch.cuda.synchronize()
        XC = XC_d.cpu().numpy().reshape(nbf, nbf, order="F")
        J = J_d.cpu().numpy().reshape(nbf, nbf, order="F")
        assert np.abs(J - J_ref).max() < 1e-10, (call, np.abs(J - J_ref).max())
        assert np.abs(XC - XC_ref).max() < 1e-10, (call, np.abs(XC - XC_ref).max())


def _noalloc(lib, phi_rows, ld, npts, cxc, cj):
    """Two calls through the C ABI on device copies; returns both (XC, J) pairs."""
    import torch
    from dftcxx_gb300 import _lib
    dev = torch.device("cuda:0")
    nbf = phi_rows.shape[0]
    buf = np.zeros((nbf, ld))
    buf[:, :npts] = phi_rows
    buf[:, npts:] = np.nan                    # the padding past npts must never be read
    phi_d = torch.from_numpy(buf).to(dev)
    cxc_d = torch.from_numpy(np.ascontiguousarray(cxc)).to(dev)
    cj_d = torch.from_numpy(np.ascontiguousarray(cj)).to(dev)
    out = []
    for _ in range(2):
        XC_d = torch.full((nbf * nbf,), float("nan"), dtype=torch.float64, device=dev)
        J_d = torch.full((nbf * nbf,), float("nan"), dtype=torch.float64, device=dev)
        _lib.check(lib.dftg_contract_noalloc(ctypes.c_void_p(phi_d.data_ptr()), ld, npts, nbf,
                                             ctypes.c_void_p(cxc_d.data_ptr()), ctypes.c_void_p(cj_d.data_ptr()),
                                             ctypes.c_void_p(XC_d.data_ptr()), ctypes.c_void_p(J_d.data_ptr()), None))
        torch.cuda.synchronize()
        out.append((XC_d.cpu().numpy().reshape(nbf, nbf, order="F"), J_d.cpu().numpy().reshape(nbf, nbf, order="F")))
    return out


def _rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def test_contract_noalloc_three_blocks_padded_rows(gpu_lib, oracle_mod):
    """130 functions: tiles (0,0) (0,1) (0,2) (1,1) (1,2) (2,2), the last block
    two functions wide; amplitude rows with stride ld = npts + 37."""
    from dftcxx_gb300 import _lib
    from dftcxx_gb300.molecule import synthetic_contraction
    from dftcxx_gb300.grid import PointGrid
    nbf, npts = 130, 6000
    pts, w, lmn, alpha, centres, P = synthetic_contraction(npts=npts, nbf=nbf, nocc=nbf // 4, seed=7)
    g = PointGrid(pts, w, centres, np.arange(nbf), lmn, np.ones(nbf, np.int32), alpha, np.ones(nbf),
                  precision="fp64")
    XC_ref = g.xc_build(P)["XC"]
    rho, wts = g.get_densities(), g.get_weights()
    L = oracle_mod.lib()
    v = np.empty_like(rho)
    e_, v_ = ctypes.c_double(), ctypes.c_double()
    for i, r in enumerate(rho):
        L.orc_lda_point(float(r), ctypes.byref(e_), ctypes.byref(v_))
        v[i] = v_.value
    phi = np.ascontiguousarray(g.get_amplitudes())
    cxc = wts * v
    cj = np.random.default_rng(8).uniform(-1.0, 1.0, npts)
    for XC, J in _noalloc(_lib.load(), phi, npts + 37, npts, cxc, cj):
        assert _rel(XC, XC_ref) <= 1e-10
        assert _rel(XC, (phi * cxc) @ phi.T) <= 1e-10
        assert _rel(J, (phi * cj) @ phi.T) <= 1e-10
        # off-diagonal blocks are written once and mirrored; diagonal blocks are
        # summed in both orders, so they agree to rounding
        assert _rel(XC, XC.T) <= 1e-14 and _rel(J, J.T) <= 1e-14
    g.close()


def test_contract_noalloc_at_the_basis_limit(gpu_lib):
    """1024 functions (the limit): one chunk of partial sums is the whole
    scratch array; rows padded to ld = npts + 8."""
    from dftcxx_gb300 import _lib
    nbf, npts = 1024, 2048
    rng = np.random.default_rng(9)
    phi = rng.normal(0.0, 1.0, (nbf, npts)) * np.exp(-rng.uniform(0, 3, (nbf, 1)))
    cxc = rng.uniform(-1.0, 0.0, npts)
    cj = rng.uniform(0.0, 1.0, npts)
    for XC, J in _noalloc(_lib.load(), phi, npts + 8, npts, cxc, cj):
        assert _rel(XC, (phi * cxc) @ phi.T) <= 1e-10
        assert _rel(J, (phi * cj) @ phi.T) <= 1e-10


def test_contract_noalloc_rejects_oversize(gpu_lib):
    import torch
    from dftcxx_gb300 import _lib
    lib = _lib.load()
    t = torch.zeros(64, dtype=torch.float64, device="cuda:0")
    p = ctypes.c_void_p(t.data_ptr())
    rc = lib.dftg_contract_noalloc(p, 8, 8, 1025, p, p, p, p, None)
    assert rc == _lib.DFTG_ERR_ARG
    assert b"no-allocation limit" in lib.dftg_last_error()
