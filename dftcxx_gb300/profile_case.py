"""Run a few device-resident grid Fock builds of one workload, for profilers.

    python -m dftcxx_gb300.profile_case [--workload benzene|h2o|decane] [--precision mixed|fp64] [--builds N]
                                        [--backward N]

Builds the grid (setup kernels), forms the core-Hamiltonian density from the
device one-electron integrals, then runs N builds through
dftg_fock_build_device on the context's stream and synchronises; with
--backward N, N backward passes (dE/dP and forces) of the last build follow.
Nothing else runs on the GPU, so a profiler sees the setup launches followed
by N identical builds (and the backward passes).
"""
import argparse
import ctypes
import sys

import numpy as np


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="benzene", choices=["benzene", "h2o", "decane"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--builds", type=int, default=2)
    ap.add_argument("--backward", type=int, default=0)
    args = ap.parse_args(argv)

    import torch
    from . import _lib
    from .build import build
    from .grid import MolecularGrid
    from .molecule import Molecule, alkane, benzene, h2o

    build()
    if args.workload == "benzene":
        Z, xyz = benzene()
        mol, grid = Molecule(Z, xyz, "p631"), (75, 11, 8)
    elif args.workload == "decane":
        Z, xyz = alkane(10)
        mol, grid = Molecule(Z, xyz, "p631"), (50, 10, 8)
    else:
        Z, xyz = h2o()
        mol, grid = Molecule(Z, xyz, "sto3g"), (32, 7, 8)
    g = MolecularGrid(mol, *grid, precision=args.precision)
    S, T, V = g.one_electron()
    lam, U = np.linalg.eigh(S)
    X = U @ np.diag(1.0 / np.sqrt(lam))
    _, Cp = np.linalg.eigh(X.T @ (T + V) @ X)
    C = X @ Cp
    P = C[:, :mol.nelec // 2] @ C[:, :mol.nelec // 2].T
    n = mol.nbf
    dP = torch.from_numpy(np.asfortranarray(P).ravel(order="F").copy()).cuda()
    dJ = torch.zeros(n * n, dtype=torch.float64, device="cuda")
    dXC = torch.zeros_like(dJ)
    dS = torch.zeros(3, dtype=torch.float64, device="cuda")
    L = _lib.load()
    for _ in range(args.builds):
        _lib.check(L.dftg_fock_build_device(g.handle, ctypes.c_void_p(dP.data_ptr()), ctypes.c_void_p(dJ.data_ptr()),
                                            ctypes.c_void_p(dXC.data_ptr()), ctypes.c_void_p(dS.data_ptr())))
    gP = torch.zeros(n * n, dtype=torch.float64, device="cuda")
    gR = torch.zeros(3 * mol.natoms, dtype=torch.float64, device="cuda")
    for _ in range(args.backward):
        _lib.check(L.dftg_backward_device(g.handle, 1.0, 1.0, ctypes.c_void_p(gP.data_ptr()),
                                          ctypes.c_void_p(gR.data_ptr())))
    torch.cuda.synchronize()
    e = g.energies()
    print("builds %d  npts %d  nbf %d  Exc %.10f  EJ %.10f  N %.10f" % (args.builds, g.grid_size, n, e["Exc"], e["EJ"],
                                                                      e["nelec"]))
    return 0


if __name__ == "__main__":
    sys.exit(main())
