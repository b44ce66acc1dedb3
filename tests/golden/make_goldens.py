"""Generate the golden fixtures of tests/golden/ from the reference itself.

Run here, where the reference sources exist: it builds oracle/_ref (the
reference's own quadrature, cubic-spline and Boys-function translation units,
compiled from their sources) and records
  * ref_lebedev.json  -- SHA-256 of the reference's Lebedev table bytes
                          (914 rows x 4 doubles) and its per-order row counts;
  * ref_spline.npz    -- seeded knots/queries and the reference's Cspline::eval
                          outputs;
  * ref_fgamma.npz    -- (m, x) grid and the reference's GammaInc::Fgamma;
  * ref_basis.json    -- SHA-256 of each reference basis file's parsed numbers;
  * oracle_h2o_scf.json -- oracle SCF energies of H2O/STO-3G/32x110 (a
                          regression record of the oracle, not a reference pin);
and, from the reference PROGRAM's own code (oracle/_ref/ref_dump*: its
unmodified grid, Hartree, XC, energy and SCF translation units compiled
against the Eigen/Boost API subset of oracle/shim):
  * ref_h2o_sto3g_32x110.npz -- the reference's SCF from its core guess to
                          |dE| <= 1e-10 (history rows E, 2tr(PH), 2tr(PJ),
                          E_xc, N; final P), and one build at that P: J, XC,
                          scalars (E_xc, E_J, 2tr(PH), E_nuc, E_tot, N before
                          and after the correction), S, T, V, H, and per point
                          w, Becke weight, rho, V_H; per atom rho_lm and U_lm;
  * ref_benzene_p631_75x302.npz -- benzene / 6-31G: the reference's SCF at
                          30 x 110 (lmax 8, |dE| <= 1e-9) gives P; one build at
                          that P on the 75 x 302 grid (ref_dump302: the 302-point
                          rule added to the reference's table) gives J, XC,
                          scalars, S, T, V, H, the per-point arrays at every
                          101st point, their full FP64 sums and the reference's
                          own phase timings on this host.
ref_dump302 is also checked to reproduce ref_dump bit for bit on H2O / 32 x 110.

Usage: python tests/golden/make_goldens.py /path/to/reference
"""
import ctypes
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle, refprog  # noqa: E402
from dftcxx_gb300.molecule import Molecule, benzene, h2o, parse_basis_dat  # noqa: E402

_dp = ctypes.POINTER(ctypes.c_double)


def main(ref_root):
    oracle.build(os.path.join(ref_root, "src"))
    R = oracle.ref_lib()
    assert R is not None, "oracle/_ref not built"

    n = R.ref_lebedev_total()
    tab = np.zeros((n, 4))
    R.ref_lebedev(tab.ctypes.data_as(_dp))
    npts = [6, 14, 26, 38, 50, 74, 86, 110, 146, 170, 194]
    offs = np.concatenate([[0], np.cumsum(npts)[:-1]])
    with open(os.path.join(HERE, "ref_lebedev.json"), "w") as f:
        json.dump({"rows": n, "sha256": hashlib.sha256(tab.tobytes()).hexdigest(), "npts": npts,
                   "weight_sums": [float(tab[o:o + k, 3].sum()) for o, k in zip(offs, npts)]}, f, indent=1)

    rng = np.random.default_rng(20261203)
    cases = {}
    for k, m in enumerate((3, 8, 32, 75)):
        x = np.sort(rng.uniform(0.0, 10.0, m))
        x = np.unique(x)
        m = x.size
        y = rng.normal(size=m)
        xq = np.concatenate([rng.uniform(-1.0, 11.0, 400), x])
        out = np.zeros(xq.size)
        R.ref_spline_eval(m, x.ctypes.data_as(_dp), y.ctypes.data_as(_dp), xq.size, xq.ctypes.data_as(_dp),
                          out.ctypes.data_as(_dp))
        cases["x%d" % k], cases["y%d" % k], cases["q%d" % k], cases["o%d" % k] = x, y, xq, out
    np.savez(os.path.join(HERE, "ref_spline.npz"), **cases)

    ms = np.arange(0, 9)
    xs = np.concatenate([[0.0, 1e-12, 1e-9, 1e-8, 2e-8, 1e-6], np.logspace(-5, 2.7, 200)])
    F = np.array([[R.ref_fgamma(int(m), float(x)) for x in xs] for m in ms])
    np.savez(os.path.join(HERE, "ref_fgamma.npz"), m=ms, x=xs, F=F)

    basis = {}
    for name in ("sto3g", "sto6g", "p321", "p631"):
        with open(os.path.join(ref_root, "basis", name + ".dat")) as f:
            data = parse_basis_dat(f.read())
        flat = np.array([v for z in sorted(data) for _, prims in data[z] for p in prims for v in p])
        basis[name] = {"sha256": hashlib.sha256(flat.tobytes()).hexdigest(), "elements": sorted(data)}
    with open(os.path.join(HERE, "ref_basis.json"), "w") as f:
        json.dump(basis, f, indent=1)

    Z, xyz = h2o()
    mol = Molecule(Z, xyz, "sto3g")
    g = oracle.OracleGrid(mol, 32, 7, 8)
    hist, mats = oracle.scf(g, tol=1e-8)
    with open(os.path.join(HERE, "oracle_h2o_scf.json"), "w") as f:
        json.dump({"config": "H2O STO-3G 32x110 lmax 8, SCF to dE<1e-8",
                   "E": [h["E"] for h in hist], "Exc": [h["Exc"] for h in hist],
                   "enuc": mats["enuc"]}, f, indent=1)


    reference_program(ref_root)


def _grid_keys(r, idx=None):
    out = {}
    for k, name in (("weights", "w"), ("becke", "becke"), ("rho", "rho"), ("potential", "V")):
        out[name] = r[k] if idx is None else r[k][idx]
    return out


def reference_program(ref_root):
    refprog.build(ref_root)
    Z, xyz = h2o()
    mol = Molecule(Z, xyz, "sto3g", "water")
    s = refprog.scf(mol, 32, 7, 8, max_iter=200, tol=1e-10)
    P = s["P"]
    r = refprog.fock_build(mol, 32, 7, 8, P, amp=True)
    r302 = refprog._run(mol.basis_name, refprog.input_text("water", "sto3g", mol.Z, mol.xyz, 32, 7, 8),
                        ["build", lambda tmp: _pfile(tmp, P)], 11)
    for k in ("J", "XC", "scalars", "rho", "potential", "weights", "becke"):
        assert np.array_equal(r[k], r302[k]), ("ref_dump302 differs from ref_dump", k)
    np.savez_compressed(os.path.join(HERE, "ref_h2o_sto3g_32x110.npz"),
                        history=s["history"], P=P, J=r["J"], XC=r["XC"], scalars=r["scalars"],
                        S=r["S"], T=r["T"], Vnuc=r["Vnuc"], H=r["H"], rho_lm=r["rho_lm"], U_lm=r["U_lm"],
                        **_grid_keys(r))

    Z, xyz = benzene()
    mol = Molecule(Z, xyz, "p631", "benzene")
    s = refprog.scf(mol, 30, 7, 8, max_iter=200, tol=1e-9)
    P = s["P"]
    r = refprog.fock_build(mol, 75, 11, 8, P)
    idx = np.arange(0, r["rho"].size, 101)
    sums = np.array([r["weights"].sum(), (r["weights"] * r["rho"]).sum(), (r["weights"] * r["potential"]).sum(),
                     (r["weights"] * r["rho"] * r["potential"]).sum(), r["becke"].sum()])
    np.savez_compressed(os.path.join(HERE, "ref_benzene_p631_75x302.npz"),
                        scf_history_30x110=s["history"], P=P, J=r["J"], XC=r["XC"], scalars=r["scalars"],
                        S=r["S"], T=r["T"], Vnuc=r["Vnuc"], H=r["H"], idx=idx, sums=sums,
                        timings_ms=r["timings_ms"], threads=np.array([os.cpu_count()]), **_grid_keys(r, idx))


def _pfile(tmp, P):
    path = os.path.join(tmp, "P.bin")
    np.asfortranarray(P).ravel(order="F").tofile(path)
    return path


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_goldens.py /path/to/reference")
    main(sys.argv[1])
