"""Failure detection without a GPU fault: a bounded device wait that expires
(an mbarrier that nothing arrives at, limit 20 ms) is reported to the host as
DFTG_ERR_TIMEOUT through the context's error flag, the kernel exits normally,
and the context stays usable: later builds reproduce the earlier ones bit for
bit."""
import numpy as np
import pytest

from dftcxx_gb300.molecule import Molecule, small_molecule

pytestmark = pytest.mark.gpu


def test_expired_wait_reports_timeout_and_context_survives(gpu_lib):
    from dftcxx_gb300 import _lib
    from dftcxx_gb300.grid import MolecularGrid
    mol = Molecule(*small_molecule("H2O"), "sto3g")
    rng = np.random.default_rng(4)
    C = rng.normal(0, 0.3, size=(mol.nbf, 5))
    P = C @ C.T
    g = MolecularGrid(mol, 16, 4, 6, precision="mixed")
    r0 = g.fock_build(P)
    L = _lib.load()
    for _ in range(2):   # the flag is cleared after each report
        rc = L.dftg_selftest_wait(g.handle, 20.0)
        assert rc == _lib.DFTG_ERR_TIMEOUT, rc
        assert b"code 99" in L.dftg_last_error()
        r1 = g.fock_build(P)
        assert np.array_equal(r1["J"], r0["J"]) and np.array_equal(r1["XC"], r0["XC"])
        assert r1["Exc"] == r0["Exc"]
    assert L.dftg_selftest_wait(g.handle, 0.0) == _lib.DFTG_ERR_ARG
    g.close()
