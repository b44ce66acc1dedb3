"""Run a few device-resident grid Fock builds of one workload, for profilers.

    python -m dftcxx_gb300.profile_case [--workload benzene|h2o|decane|synthetic] [--precision mixed|fp64]
                                        [--builds N] [--backward N] [--scf N] [--points N] [--nbf N]

Builds the grid (setup kernels), forms the core-Hamiltonian density from the
device one-electron integrals, then runs N builds through
dftg_fock_build_device on the context's stream and synchronises; with
--backward N, N backward passes (dE/dP and forces) of the last build follow.
Nothing else runs on the GPU, so a profiler sees the setup launches followed
by N identical builds (and the backward passes).  --scf N: instead, the device
SCF driver's set-up and N iterations (one conditional-graph launch; with
--scf-step one graph launch per iteration, for profilers).
--workload synthetic: the seeded point-set workload (--points, --nbf; default
2,000,000 x 512) through dftg_xc_build_device.
--workload batch: --nmol jittered small molecules (H2 .. C6H6, STO-3G and
6-31G, 50 x 194, lmax 8, mixed) built --builds times as one batch
(--batch-mode persistent or graph; the first build runs eagerly, the second
captures the graph, the rest replay it).
"""
import argparse
import ctypes
import sys

import numpy as np


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="benzene", choices=["benzene", "h2o", "decane", "synthetic", "batch"])
    ap.add_argument("--nmol", type=int, default=64)
    ap.add_argument("--batch-mode", default="persistent", choices=["persistent", "graph"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--builds", type=int, default=2)
    ap.add_argument("--backward", type=int, default=0)
    ap.add_argument("--scf", type=int, default=0)
    ap.add_argument("--scf-step", action="store_true", help="run the SCF iterations as one graph launch each")
    ap.add_argument("--points", type=int, default=2_000_000)
    ap.add_argument("--nbf", type=int, default=512)
    args = ap.parse_args(argv)

    import torch
    from . import _lib
    from .build import build
    from .grid import MolecularGrid
    from .molecule import Molecule, alkane, benzene, h2o

    build()
    if args.workload == "synthetic":
        return _synthetic(args)
    if args.workload == "batch":
        return _batch(args)
    if args.workload == "benzene":
        Z, xyz = benzene()
        mol, grid = Molecule(Z, xyz, "p631"), (75, 11, 8)
    elif args.workload == "decane":
        Z, xyz = alkane(10)
        mol, grid = Molecule(Z, xyz, "p631"), (50, 10, 8)
    else:
        Z, xyz = h2o()
        mol, grid = Molecule(Z, xyz, "sto3g"), (32, 7, 8)
    if args.scf:
        from .grid import DeviceSCF
        d = DeviceSCF(mol, *grid, precision=args.precision, tol=0.0, min_iter=args.scf, max_iter=args.scf)
        if args.scf_step:
            for _ in range(args.scf):
                E, _ = d.step()
            d.iterations = args.scf
        else:
            E = d.run()
        torch.cuda.synchronize()
        print("scf iterations %d  E %.10f  diag %s" % (d.iterations, E, d.diagnostics()))
        return 0
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


def _synthetic(args):
    import torch
    from . import _lib
    from .grid import PointGrid
    from .molecule import synthetic_contraction
    pts, w, lmn, alpha, centres, P = synthetic_contraction(npts=args.points, nbf=args.nbf, nocc=min(128, args.nbf))
    n = args.nbf
    g = PointGrid(pts, w, centres, np.arange(n), lmn, np.ones(n, np.int32), alpha, np.ones(n),
                  precision=args.precision)
    dP = torch.from_numpy(np.asfortranarray(P).ravel(order="F").copy()).cuda()
    XC = torch.zeros(n * n, dtype=torch.float64, device="cuda")
    sc = torch.zeros(2, dtype=torch.float64, device="cuda")
    L = _lib.load()
    for _ in range(args.builds):
        _lib.check(L.dftg_xc_build_device(g.handle, ctypes.c_void_p(dP.data_ptr()), ctypes.c_void_p(XC.data_ptr()),
                                          ctypes.c_void_p(sc.data_ptr())))
    torch.cuda.synchronize()
    print("synthetic builds %d  npts %d  nbf %d  Exc %.10f" % (args.builds, args.points, n, float(sc[0])))
    return 0


def _batch(args):
    import torch
    from .grid import Batch, MolecularGrid
    from .molecule import Molecule, small_molecule
    names = ["H2", "LiH", "H2O", "NH3", "CH4", "N2", "CO", "C2H6", "C6H6"]
    rng = np.random.default_rng(20261204)
    grids, Ps = [], []
    for i in range(args.nmol):
        Z, xyz = small_molecule(names[i % len(names)])
        xyz = np.asarray(xyz, dtype=float) + rng.normal(0.0, 0.05, size=(len(Z), 3))
        mol = Molecule(Z, xyz, "sto3g" if (i // len(names)) % 2 == 0 else "p631")
        grids.append(MolecularGrid(mol, 50, 10, 8, precision="mixed"))
        C = rng.normal(0, 0.2, size=(mol.nbf, max(1, mol.nelec // 2)))
        Ps.append(torch.from_numpy(np.asfortranarray(C @ C.T).ravel(order="F").copy()).cuda())
    outs = [torch.zeros(g.nbf * g.nbf, dtype=torch.float64, device="cuda") for g in grids]
    b = Batch(grids, mode=args.batch_mode)
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()
    for _ in range(args.builds):
        b.build(Ps, outs, None, None, stream=stream.cuda_stream)
    b.status()
    print("batch builds %d  molecules %d  persistent %s" % (args.builds, args.nmol, b.persistent_active()))
    b.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
