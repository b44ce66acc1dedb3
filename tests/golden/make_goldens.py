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
                          regression record of the oracle, not a reference pin).

Usage: python tests/golden/make_goldens.py [/path/to/reference]
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

from oracle import oracle  # noqa: E402
from dftcxx_gb300.molecule import Molecule, h2o, parse_basis_dat  # noqa: E402

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


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
