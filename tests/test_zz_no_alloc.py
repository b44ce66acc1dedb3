"""dftg_contract_noalloc: the XC / J contraction for callers that may not
allocate device memory while they serve (their framework owns all GPU memory,
or they run under a fixed device-memory budget).

The entry point is called through the C ABI on caller-owned device buffers,
twice in a row (the second call reuses the static scratch the first one left
behind), and each result is checked against the context's own entry points
(dftg_calculate_hartree_potential and dftg_calculate_xc) to 1e-10.  This file
is collected last so that a stop-at-first-failure run has already run every
other test."""
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


def test_contract_noalloc_rejects_oversize(gpu_lib):
    import torch
    from dftcxx_gb300 import _lib
    lib = _lib.load()
    t = torch.zeros(64, dtype=torch.float64, device="cuda:0")
    p = ctypes.c_void_p(t.data_ptr())
    rc = lib.dftg_contract_noalloc(p, 8, 8, 1025, p, p, p, p, None)
    assert rc == _lib.DFTG_ERR_ARG
    assert b"no-allocation limit" in lib.dftg_last_error()
