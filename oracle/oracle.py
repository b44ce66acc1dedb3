"""ctypes wrapper over the CPU FP64 oracle (``oracle/dftg_oracle.c``).

TEST INFRASTRUCTURE: only tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of bench.py may import this module.  It is the checker, never
the product: the product path (``dftcxx_gb300``) does not import it.

Also exposes the reference's own dependency-free translation units compiled
into ``oracle/_ref/`` (Lebedev table, cubic spline, Boys function) when that
library has been built (it needs the reference sources at build time).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libdftg_oracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libdftcxx_ref.so")

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_lib = None
_ref = None


def build(ref_src=None):
    """Compile the oracle; with ref_src (the reference's src/ folder), also the
    reference's dependency-free units into oracle/_ref."""
    subprocess.check_call(["make", "-s", "-C", HERE, "all"])
    if ref_src and os.path.isdir(ref_src):
        subprocess.check_call(["make", "-s", "-C", HERE, "ref", "REFSRC=" + ref_src])


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.orc_create.restype = ctypes.c_void_p
        L.orc_create.argtypes = [ctypes.c_int, _ip, _dp, ctypes.c_int, _ip, _ip, _ip, _dp, _dp,
                                 ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.orc_destroy.argtypes = [ctypes.c_void_p]
        L.orc_grid_size.restype = ctypes.c_long
        L.orc_grid_size.argtypes = [ctypes.c_void_p]
        for name in ("orc_get_weights", "orc_get_becke_weights", "orc_get_densities", "orc_get_positions",
                     "orc_get_potential", "orc_get_radii", "orc_get_amplitudes", "orc_get_U", "orc_get_rho_lm",
                     "orc_set_density"):
            getattr(L, name).argtypes = [ctypes.c_void_p, _dp]
        L.orc_calculate_density.restype = ctypes.c_double
        L.orc_calculate_density.argtypes = [ctypes.c_void_p]
        L.orc_correct_densities.restype = ctypes.c_double
        L.orc_correct_densities.argtypes = [ctypes.c_void_p]
        L.orc_xc.restype = ctypes.c_double
        L.orc_xc.argtypes = [ctypes.c_void_p, _dp, _dp]
        L.orc_hartree.argtypes = [ctypes.c_void_p, _dp]
        L.orc_one_electron.argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
        L.orc_nuclear_repulsion.restype = ctypes.c_double
        L.orc_nuclear_repulsion.argtypes = [ctypes.c_void_p]
        L.orc_eri.restype = ctypes.c_double
        L.orc_eri.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.orc_eri_list.restype = None
        L.orc_eri_list.argtypes = [ctypes.c_void_p, _dp]
        L.orc_eri_coulomb.restype = None
        L.orc_eri_coulomb.argtypes = [ctypes.c_void_p, _dp, _dp]
        L.orc_fgamma.restype = ctypes.c_double
        L.orc_fgamma.argtypes = [ctypes.c_int, ctypes.c_double]
        L.orc_ylm.restype = ctypes.c_double
        L.orc_ylm.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double]
        L.orc_spline_eval.argtypes = [ctypes.c_int, _dp, _dp, ctypes.c_int, _dp, _dp]
        L.orc_lda_point.argtypes = [ctypes.c_double, _dp, _dp]
        L.orc_gto_norm.restype = ctypes.c_double
        L.orc_gto_norm.argtypes = [ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.orc_poisson_matrix.argtypes = [ctypes.c_int, _dp, _dp]
        L.orc_points_xc.restype = ctypes.c_double
        L.orc_points_xc.argtypes = [ctypes.c_long, _dp, _dp, ctypes.c_int, _dp, _ip, _ip, _ip, _dp, _dp, _dp,
                                    ctypes.c_int, _dp, _dp]
        L.orc_num_threads.restype = ctypes.c_int
        L.orc_set_sample_stride.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.orc_shard_density.restype = ctypes.c_double
        L.orc_shard_density.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int, ctypes.c_int]
        L.orc_shard_blob_doubles.restype = ctypes.c_long
        L.orc_shard_blob_doubles.argtypes = [ctypes.c_void_p]
        L.orc_shard_multipoles.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_int, _dp]
        L.orc_shard_finish.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.c_int, ctypes.c_int, _dp, _dp, _dp]
        L.orc_get_timings.argtypes = [ctypes.c_void_p, _dp]
        _lib = L
    return _lib


def ref_lib():
    """The reference's own quadrature/cspline/gamma units, or None."""
    global _ref
    if _ref is None and os.path.exists(REF_PATH):
        R = ctypes.CDLL(REF_PATH)
        R.ref_lebedev_total.restype = ctypes.c_int
        R.ref_lebedev.argtypes = [_dp]
        R.ref_spline_eval.argtypes = [ctypes.c_int, _dp, _dp, ctypes.c_int, _dp, _dp]
        R.ref_fgamma.restype = ctypes.c_double
        R.ref_fgamma.argtypes = [ctypes.c_int, ctypes.c_double]
        _ref = R
    return _ref


def _p(a, ct=_dp):
    return a.ctypes.data_as(ct)


class OracleGrid:
    """CPU FP64 restatement of MolecularGrid + the XC/energy part of DFT."""

    def __init__(self, mol, nrad, lebedev_order, lmax):
        L = lib()
        self.mol = mol
        self._keep = [np.ascontiguousarray(mol.Z, dtype=np.int32),
                      np.ascontiguousarray(mol.xyz, dtype=np.float64),
                      np.ascontiguousarray(mol.bf_atom, dtype=np.int32),
                      np.ascontiguousarray(mol.bf_lmn, dtype=np.int32),
                      np.ascontiguousarray(mol.bf_nprim, dtype=np.int32),
                      np.ascontiguousarray(mol.prim_alpha, dtype=np.float64),
                      np.ascontiguousarray(mol.prim_coef, dtype=np.float64)]
        Z, xyz, ba, bl, bn, pa, pc = self._keep
        self.h = L.orc_create(mol.natoms, _p(Z, _ip), _p(xyz), mol.nbf, _p(ba, _ip), _p(bl, _ip), _p(bn, _ip),
                              _p(pa), _p(pc), nrad, lebedev_order, lmax)
        if not self.h:
            raise ValueError("oracle: invalid grid parameters")
        self.nbf = mol.nbf
        self.nrad, self.lmax = nrad, lmax
        self.npts = L.orc_grid_size(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def _get(self, name, shape):
        out = np.empty(shape, dtype=np.float64)
        getattr(lib(), name)(self.h, _p(out))
        return out

    def weights(self):
        return self._get("orc_get_weights", self.npts)

    def becke_weights(self):
        return self._get("orc_get_becke_weights", self.npts)

    def densities(self):
        return self._get("orc_get_densities", self.npts)

    def positions(self):
        return self._get("orc_get_positions", (self.npts, 3))

    def potential(self):
        return self._get("orc_get_potential", self.npts)

    def radii(self):
        return self._get("orc_get_radii", self.nrad)

    def amplitudes(self):
        """[npts, nbf] (the reference's nbf x npts column-major matrix)."""
        return self._get("orc_get_amplitudes", (self.npts, self.nbf))

    def U_lm(self):
        return self._get("orc_get_U", (self.mol.natoms, self.nrad, (self.lmax + 1) ** 2))

    def rho_lm(self):
        return self._get("orc_get_rho_lm", (self.mol.natoms, self.nrad, (self.lmax + 1) ** 2))

    def set_density(self, P):
        P = np.asfortranarray(P, dtype=np.float64)
        lib().orc_set_density(self.h, P.ctypes.data_as(_dp))

    def correct_densities(self):
        return lib().orc_correct_densities(self.h)

    def calculate_density(self):
        return lib().orc_calculate_density(self.h)

    def hartree(self):
        J = np.zeros((self.nbf, self.nbf), order="F")
        lib().orc_hartree(self.h, J.ctypes.data_as(_dp))
        return np.ascontiguousarray(J)

    def xc(self, want_v=False):
        XC = np.zeros((self.nbf, self.nbf), order="F")
        v = np.zeros(self.npts) if want_v else None
        exc = lib().orc_xc(self.h, XC.ctypes.data_as(_dp), _p(v) if want_v else None)
        XC = np.ascontiguousarray(XC)
        return (XC, exc, v) if want_v else (XC, exc)

    def one_electron(self):
        n = self.nbf
        S, T, V = (np.zeros((n, n), order="F") for _ in range(3))
        lib().orc_one_electron(self.h, S.ctypes.data_as(_dp), T.ctypes.data_as(_dp), V.ctypes.data_as(_dp))
        return np.ascontiguousarray(S), np.ascontiguousarray(T), np.ascontiguousarray(V)

    def nuclear_repulsion(self):
        return lib().orc_nuclear_repulsion(self.h)

    def eri(self, i, j, k, l):
        """Contracted (ij|kl), Integrator::repulsion (integrals.cpp:185-466)."""
        return lib().orc_eri(self.h, i, j, k, l)

    def eri_list(self):
        """Every unique (ij|kl) at the reference's teindex position (integrals.cpp:470-486)."""
        npair = self.nbf * (self.nbf + 1) // 2
        out = np.zeros(npair * (npair + 1) // 2)
        lib().orc_eri_list(self.h, _p(out))
        return out

    def eri_coulomb(self, P):
        """J_ij = sum_kl P_kl (ij|kl), DFT::calculate_hartree_potential_te_int (dft.cpp:452-477)."""
        P = np.asfortranarray(P, dtype=np.float64)
        J = np.zeros((self.nbf, self.nbf), order="F")
        lib().orc_eri_coulomb(self.h, P.ctypes.data_as(_dp), J.ctypes.data_as(_dp))
        return np.ascontiguousarray(J)

    def set_sample_stride(self, stride):
        """Timing-only mode: point loops of the cross-atom potential, J and XC
        visit every stride-th point (results are then NOT the full build)."""
        lib().orc_set_sample_stride(self.h, int(stride))

    def timings(self):
        """Wall times of the last build: [multipole+Poisson, cross-atom V, J, XC]."""
        return self._get("orc_get_timings", 4)

    def fock_build(self, P):
        """One grid Fock build at fixed P: set_density, correct_densities,
        Hartree J, XC; returns a dict (dft.cpp:361-365, 377-447)."""
        self.set_density(P)
        c = self.correct_densities()
        J = self.hartree()
        XC, exc = self.xc()
        return {"J": J, "XC": XC, "Exc": exc, "scale": c, "nelec": self.calculate_density()}


class OracleShard:
    """The cells [first_cell, first_cell + ncells) of an oracle grid, with the
    interface of dftcxx_gb300.shard's backends (density / multipoles /
    finish): the CPU stand-in of one rank in checks of the sharded build."""

    def __init__(self, mol, nrad, lebedev_order, lmax, first_cell, ncells):
        self.grid = OracleGrid(mol, nrad, lebedev_order, lmax)
        self.first_cell, self.ncells = first_cell, ncells
        self.blob_per_cell = int(lib().orc_shard_blob_doubles(self.grid.h))
        self.nbf = mol.nbf

    def density(self, P):
        P = np.asfortranarray(P, dtype=np.float64)
        return lib().orc_shard_density(self.grid.h, _p(P), self.first_cell, self.ncells)

    def multipoles(self, total):
        blob = np.zeros(self.blob_per_cell * self.ncells)
        lib().orc_shard_multipoles(self.grid.h, float(total), self.first_cell, self.ncells, _p(blob))
        return blob

    def finish(self, blob_all, P):
        n = self.nbf
        blob_all = np.ascontiguousarray(blob_all, dtype=np.float64)
        P = np.asfortranarray(P, dtype=np.float64)
        J = np.zeros((n, n), order="F")
        XC = np.zeros((n, n), order="F")
        sc = np.zeros(3)
        lib().orc_shard_finish(self.grid.h, _p(blob_all), _p(P), self.first_cell, self.ncells, _p(J), _p(XC), _p(sc))
        return np.ascontiguousarray(J), np.ascontiguousarray(XC), sc


def energy(P, H, J, enuc, exc):
    """DFT::calculate_energy, dft.cpp:441-447."""
    e1 = 2.0 * np.trace(P @ H)
    ej = 2.0 * np.trace(P @ J)
    return e1 + ej + enuc + exc, e1, ej


def scf(grid, max_iter=100, tol=1e-8, min_iter=3, alpha=0.5):
    """Reference SCF (dft.cpp:84-142, 160-227, 300-366) on the oracle grid.

    Canonical orthogonalisation X = U diag(lambda^-1/2); F = H + 2J + XC;
    P = C_occ C_occ^T; linear damping P <- (1-alpha) P_new + alpha P after the
    first density.  Returns the list of per-iteration records."""
    mol = grid.mol
    S, T, Vn = grid.one_electron()
    H = T + Vn
    enuc = grid.nuclear_repulsion()
    lam, U = np.linalg.eigh(S)
    X = U @ np.diag(1.0 / np.sqrt(lam))
    nocc = mol.nelec // 2
    n = mol.nbf
    J = np.zeros((n, n))
    XC = np.zeros((n, n))
    P = None

    def density(P):
        F = H + 2.0 * J + XC
        e, Cp = np.linalg.eigh(X.T @ F @ X)
        C = X @ Cp
        Pn = C[:, :nocc] @ C[:, :nocc].T
        return Pn if P is None else (1.0 - alpha) * Pn + alpha * P

    # construct_matrices: first density from H, then J and the energy
    P = density(P)
    grid.set_density(P)
    grid.correct_densities()
    J = grid.hartree()
    exc = 0.0
    et, _, _ = energy(P, H, J, enuc, exc)
    hist = []
    old = et
    it = 0
    diff = 1.0
    while diff > tol or it < min_iter:
        it += 1
        P = density(P)
        grid.set_density(P)
        grid.correct_densities()
        J = grid.hartree()
        XC, exc = grid.xc()
        et, e1, ej = energy(P, H, J, enuc, exc)
        hist.append({"iter": it, "E": et, "Exc": exc, "EJ": ej, "E1": e1, "P": P.copy(), "J": J.copy(),
                     "XC": XC.copy(), "nelec": grid.calculate_density()})
        diff = abs(et - old)
        old = et
        if it >= max_iter:
            break
    return hist, {"S": S, "T": T, "V": Vn, "H": H, "enuc": enuc}


def points_xc(xyz, w, centres, bf_centre, lmn, nprim, alpha, coef, P, stride=1, want_rho=True, want_xc=True):
    """Explicit-point XC step (orc_points_xc): returns (E_xc, rho, XC)."""
    L = lib()
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    w = np.ascontiguousarray(w, dtype=np.float64)
    centres = np.ascontiguousarray(centres, dtype=np.float64)
    bc = np.ascontiguousarray(bf_centre, dtype=np.int32)
    lmn = np.ascontiguousarray(lmn, dtype=np.int32)
    nprim = np.ascontiguousarray(nprim, dtype=np.int32)
    alpha = np.ascontiguousarray(alpha, dtype=np.float64)
    coef = np.ascontiguousarray(coef, dtype=np.float64)
    P = np.ascontiguousarray(P, dtype=np.float64)
    n, nbf = len(w), len(bc)
    rho = np.zeros(n) if want_rho else None
    XC = np.zeros((nbf, nbf)) if want_xc else None
    e = L.orc_points_xc(n, _p(xyz), _p(w), nbf, _p(centres), _p(bc, _ip), _p(lmn, _ip), _p(nprim, _ip), _p(alpha),
                        _p(coef), _p(P), int(stride), _p(rho) if rho is not None else None,
                        _p(XC) if XC is not None else None)
    return e, rho, XC
