"""CPU checks of the oracle: pinned against the reference's own compiled
translation units (golden fixtures made by tests/golden/make_goldens.py) and
against analytic known answers.  No GPU needed."""
import ctypes
import hashlib
import json
import math
import os

import numpy as np
import pytest

from dftcxx_gb300.molecule import Molecule, h2o, small_molecule, parse_basis_dat, load_basis

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
_dp = ctypes.POINTER(ctypes.c_double)


def _lebedev_table():
    import re
    path = os.path.join(os.path.dirname(GOLD), "..", "dftcxx_gb300", "csrc", "lebedev_data.h")
    rows = re.findall(r"\{([-0-9., ]+)\},", open(path).read())
    return np.array([[float(v) for v in r.split(",")] for r in rows])


def test_lebedev_table_is_the_references():
    """First 914 rows (orders 0..10) are byte-identical to quadrature.h's table."""
    gold = json.load(open(os.path.join(GOLD, "ref_lebedev.json")))
    tab = _lebedev_table()
    assert tab.shape == (914 + 302, 4)
    assert hashlib.sha256(np.ascontiguousarray(tab[:914]).tobytes()).hexdigest() == gold["sha256"]


def test_lebedev_live_reference_if_built(oracle_mod):
    R = oracle_mod.ref_lib()
    if R is None:
        pytest.skip("oracle/_ref not built (needs the reference sources)")
    tab = np.zeros((R.ref_lebedev_total(), 4))
    R.ref_lebedev(tab.ctypes.data_as(_dp))
    assert np.array_equal(tab, _lebedev_table()[:914])


@pytest.mark.parametrize("order,degree", [(4, 11), (7, 17), (10, 23), (11, 29)])
def test_lebedev_exactness(order, degree):
    """Each rule integrates monomials x^a y^b z^c, a+b+c <= degree, exactly (to
    the 12-decimal rounding of the table)."""
    npts = [6, 14, 26, 38, 50, 74, 86, 110, 146, 170, 194, 302]
    off = sum(npts[:order])
    t = _lebedev_table()[off:off + npts[order]]
    x, y, z, w = t.T
    assert abs(w.sum() - 1.0) < 1e-10
    for a in range(0, degree + 1, 2):
        for b in range(0, degree + 1 - a, 2):
            for c in range(0, degree + 1 - a - b, 2):
                exact = (math.gamma((a + 1) / 2) * math.gamma((b + 1) / 2) * math.gamma((c + 1) / 2) /
                         math.gamma((a + b + c + 3) / 2)) / (4 * math.pi) * 2
                got = np.sum(w * x ** a * y ** b * z ** c)
                assert abs(got - exact) < 5e-10, (a, b, c, got, exact)


def test_spline_matches_reference(oracle_mod):
    d = np.load(os.path.join(GOLD, "ref_spline.npz"))
    L = oracle_mod.lib()
    k = 0
    while "x%d" % k in d:
        x, y, q, o = (np.ascontiguousarray(d[n + str(k)]) for n in "xyqo")
        out = np.zeros(q.size)
        L.orc_spline_eval(x.size, x.ctypes.data_as(_dp), y.ctypes.data_as(_dp), q.size, q.ctypes.data_as(_dp),
                          out.ctypes.data_as(_dp))
        assert np.array_equal(out, o), k    # bit-identical to Cspline::eval
        k += 1
    assert k == 4


def test_fgamma_matches_reference(oracle_mod):
    d = np.load(os.path.join(GOLD, "ref_fgamma.npz"))
    L = oracle_mod.lib()
    for i, m in enumerate(d["m"]):
        for j, x in enumerate(d["x"]):
            ref = d["F"][i, j]
            got = L.orc_fgamma(int(m), float(x))
            assert abs(got - ref) <= 1e-13 * abs(ref), (m, x, got, ref)


def test_basis_data_is_the_references():
    gold = json.load(open(os.path.join(GOLD, "ref_basis.json")))
    for name, g in gold.items():
        data = load_basis(name)
        flat = np.array([v for z in sorted(data) for _, prims in data[z] for p in prims for v in p])
        assert hashlib.sha256(flat.tobytes()).hexdigest() == g["sha256"], name
        assert sorted(data) == g["elements"]


def test_ylm_against_closed_forms(oracle_mod):
    L = oracle_mod.lib()
    rng = np.random.default_rng(1)
    for _ in range(50):
        v = rng.normal(size=3)
        x, y, z = v / np.linalg.norm(v)
        c = 1 / math.sqrt(4 * math.pi)
        checks = {
            (0, 0): c,
            (1, 0): math.sqrt(3) * c * z,
            (1, 1): -math.sqrt(3) * c * x,          # Condon-Shortley phase
            (1, -1): -math.sqrt(3) * c * y,
            (2, 0): math.sqrt(5) * c * 0.5 * (3 * z * z - 1),
            (2, 2): math.sqrt(5) * c * math.sqrt(3) / 2 * (x * x - y * y),
            (2, -2): math.sqrt(5) * c * math.sqrt(3) * x * y,
        }
        for (l, m), ref in checks.items():
            assert abs(L.orc_ylm(l, m, 2 * x, 2 * y, 2 * z) - ref) < 1e-14, (l, m)


def test_ylm_orthonormal_on_lebedev():
    """Y_lm (reference convention) are orthonormal under the 302-point rule up to l = 8."""
    from oracle import oracle as om
    L = om.lib()
    t = _lebedev_table()[914:]
    lms = [(l, m) for l in range(9) for m in range(-l, l + 1)]
    Y = np.array([[L.orc_ylm(l, m, *p[:3]) for p in t] for l, m in lms])
    G = (Y * t[:, 3]) @ Y.T * 4 * math.pi
    assert np.abs(G - np.eye(len(lms))).max() < 1e-9


def test_lda_known_answers(oracle_mod):
    """Slater + VWN point values against the same formulas in high precision."""
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.dps = 40
    L = oracle_mod.lib()

    def ref(rho):
        rho = mpmath.mpf(rho)
        pi = mpmath.pi
        fac = mpmath.mpf(-2.25) * mpmath.mpf(2) / 3 * (mpmath.mpf(3) / 4 / pi) ** (mpmath.mpf(1) / 3)
        da = rho / 2
        ex = 2 * fac * da ** (mpmath.mpf(4) / 3)
        vx = mpmath.mpf(4) / 3 * fac * da ** (mpmath.mpf(1) / 3)
        A, x0, b, c = (mpmath.mpf(s) for s in ("0.0310907", "-0.10498", "3.72744", "12.9352"))
        x = (mpmath.mpf(3) / 4 / pi / rho) ** (mpmath.mpf(1) / 6)
        X = lambda t: t * t + b * t + c  # noqa: E731
        q = mpmath.sqrt(4 * c - b * b)
        eps = A * (mpmath.log(x * x / X(x)) - b * (x0 / X(x0)) * mpmath.log((x - x0) ** 2 / X(x))
                   + (2 * b / q) * (1 - x0 * (2 * x0 + b) / X(x0)) * mpmath.atan(q / (2 * x + b)))
        deps = mpmath.diff(lambda t: A * (mpmath.log(t * t / X(t)) - b * (x0 / X(x0)) * mpmath.log((t - x0) ** 2 / X(t))
                                          + (2 * b / q) * (1 - x0 * (2 * x0 + b) / X(x0)) * mpmath.atan(q / (2 * t + b))), x)
        return float(ex + eps * rho), float(vx + eps - x / 6 * deps)

    for rho in (1e-9, 1e-6, 1e-3, 0.1, 1.0, 10.0, 300.0):
        e, v = ctypes.c_double(), ctypes.c_double()
        L.orc_lda_point(rho, ctypes.byref(e), ctypes.byref(v))
        re, rv = ref(rho)
        assert abs(e.value - re) <= 1e-12 * abs(re), rho
        assert abs(v.value - rv) <= 1e-12 * abs(rv), rho
    e, v = ctypes.c_double(), ctypes.c_double()
    L.orc_lda_point(0.9e-10, ctypes.byref(e), ctypes.byref(v))   # below both 1e-10 cut-offs
    assert e.value == 0.0 and v.value == 0.0


def test_grid_overlap_and_charge(oracle_mod):
    """Phi^T diag(w) Phi reproduces the analytic overlap; the corrected density
    integrates to the electron count (moleculargrid.cpp:132-146)."""
    Z, xyz = h2o()
    mol = Molecule(Z, xyz, "sto3g")
    g = oracle_mod.OracleGrid(mol, 32, 7, 8)
    S, _, _ = g.one_electron()
    phi, w = g.amplitudes(), g.weights()
    assert np.abs(phi.T @ (w[:, None] * phi) - S).max() < 2e-4
    assert np.abs(np.diag(S) - 1.0).max() < 1e-6
    rng = np.random.default_rng(2)
    C = rng.normal(size=(mol.nbf, 5))
    g.set_density(C @ C.T)
    c = g.correct_densities()
    assert c > 0
    assert abs(g.calculate_density() - mol.nelec) < 1e-10


def _eri_ssss(a, A, b, B, c, C, d, D):
    p, q = a + b, c + d
    P = (a * A + b * B) / p
    Q = (c * C + d * D) / q
    T = p * q / (p + q) * np.sum((P - Q) ** 2)
    F0 = 1.0 if T < 1e-15 else 0.5 * math.sqrt(math.pi / T) * math.erf(math.sqrt(T))
    return (2 * math.pi ** 2.5 / (p * q * math.sqrt(p + q)) * math.exp(-a * b / p * np.sum((A - B) ** 2))
            * math.exp(-c * d / q * np.sum((C - D) ** 2)) * F0)


def _eri_s_basis(mol):
    """(ij|kl) for an s-only basis (contracted, normalised as cgf.cpp:102-114)."""
    from oracle.oracle import lib
    L = lib()
    funcs = []
    off = 0
    for i in range(mol.nbf):
        n = mol.bf_nprim[i]
        prims = [(mol.prim_alpha[off + k], mol.prim_coef[off + k] * L.orc_gto_norm(mol.prim_alpha[off + k], 0, 0, 0))
                 for k in range(n)]
        funcs.append((mol.xyz[mol.bf_atom[i]], prims))
        off += n
    nb = mol.nbf
    G = np.zeros((nb,) * 4)
    for i in range(nb):
        for j in range(nb):
            for k in range(nb):
                for l in range(nb):
                    s = 0.0
                    for a, ca in funcs[i][1]:
                        for b, cb in funcs[j][1]:
                            for c, cc in funcs[k][1]:
                                for d, cd in funcs[l][1]:
                                    s += ca * cb * cc * cd * _eri_ssss(a, funcs[i][0], b, funcs[j][0], c, funcs[k][0],
                                                                       d, funcs[l][0])
                    G[i, j, k, l] = s
    return G


def test_becke_poisson_J_vs_analytic_eri(oracle_mod):
    """Grid J (Becke-Poisson) against J_ij = sum_kl P_kl (ij|kl) (dft.cpp:452-477)
    for H2 / STO-3G, the reference's two Hartree routes."""
    Z, xyz = small_molecule("H2")
    mol = Molecule(Z, xyz, "sto3g")
    g = oracle_mod.OracleGrid(mol, 75, 11, 8)
    P = np.array([[0.3, 0.25], [0.25, 0.3]])
    g.set_density(P)
    g.correct_densities()
    J = g.hartree()
    # the grid density is rescaled to integrate to N: apply the same factor
    S, _, _ = g.one_electron()
    c = mol.nelec / (2 * np.sum(P * S))
    G = _eri_s_basis(mol)
    Jeri = np.einsum("kl,ijkl->ij", c * P, G)
    assert np.abs(J - Jeri).max() < 2e-4, np.abs(J - Jeri).max()


def test_oracle_scf_golden(oracle_mod):
    gold = json.load(open(os.path.join(GOLD, "oracle_h2o_scf.json")))
    Z, xyz = h2o()
    mol = Molecule(Z, xyz, "sto3g")
    g = oracle_mod.OracleGrid(mol, 32, 7, 8)
    hist, mats = oracle_mod.scf(g, tol=1e-8)
    assert len(hist) == len(gold["E"])
    assert np.abs(np.array([h["E"] for h in hist]) - gold["E"]).max() < 1e-9
    assert abs(mats["enuc"] - gold["enuc"]) < 1e-12
    assert abs(hist[-1]["nelec"] - 10.0) < 1e-9


def test_points_xc_matches_numpy(oracle_mod):
    """Explicit-point XC step of the oracle against a numpy restatement on a
    small synthetic set: amplitudes from the normalised primitives, rho =
    2 phi^T P phi, the oracle's LDA point function, XC = phi^T diag(w v) phi."""
    from dftcxx_gb300.molecule import synthetic_contraction
    pts, w, lmn, alpha, centres, P = synthetic_contraction(npts=400, nbf=10, nocc=3, box=6.0)
    nbf = len(alpha)
    L = oracle_mod.lib()
    phi = np.zeros((len(w), nbf))
    for i in range(nbf):
        d = pts - centres[i]
        norm = L.orc_gto_norm(float(alpha[i]), int(lmn[i, 0]), int(lmn[i, 1]), int(lmn[i, 2]))
        phi[:, i] = norm * d[:, 0] ** lmn[i, 0] * d[:, 1] ** lmn[i, 1] * d[:, 2] ** lmn[i, 2] * \
            np.exp(-alpha[i] * (d * d).sum(axis=1))
    rho = 2.0 * np.einsum("pi,ij,pj->p", phi, P, phi)
    e = np.zeros(len(w))
    v = np.zeros(len(w))
    ex, vx = ctypes.c_double(), ctypes.c_double()
    for p in range(len(w)):
        L.orc_lda_point(float(rho[p]), ctypes.byref(ex), ctypes.byref(vx))
        e[p], v[p] = ex.value, vx.value
    XC = phi.T @ (phi * (w * v)[:, None])
    got_e, got_rho, got_xc = oracle_mod.points_xc(pts, w, centres, np.arange(nbf), lmn, np.ones(nbf, np.int32), alpha,
                                                  np.ones(nbf), P)
    np.testing.assert_allclose(got_rho, rho, rtol=1e-13, atol=1e-300)
    assert abs(got_e - float(w @ e)) <= 1e-12 * abs(float(w @ e))
    np.testing.assert_allclose(got_xc, XC, rtol=1e-12, atol=1e-14 * np.abs(XC).max())
