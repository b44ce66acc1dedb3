"""Python mirror of DFTCXX's MolecularGrid / DFT call surface over the C ABI.

``MolecularGrid`` keeps the reference's method names and argument meanings
(moleculargrid.h:84-167); ``DFT`` keeps ``scf()`` and the energy bookkeeping
(dft.h:83-91, dft.cpp:84-142, 300-366, 441-447).  Every grid operation runs in
``libdftg.so``; the host side only moves nbf x nbf matrices and runs the small
eigen-solves of the SCF driver.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import check

_dp = ctypes.POINTER(ctypes.c_double)


def _ptr(a):
    return a.ctypes.data_as(_dp)


class MolecularGrid:
    """Becke-partitioned Gauss-Chebyshev x Lebedev grid on one GPU.

    ``precision``: "fp64" (every step in FP64) or "mixed" (split-precision
    contractions, FP64 reductions)."""

    def __init__(self, mol, radial_points=15, lebedev_order=7, lmax=8, precision="fp64", device=0, cells=None):
        """cells: (first_cell, ncells) for a context over part of the molecule's
        fuzzy cells (an atom-cell shard, built with dftcxx_gb300.shard)."""
        L = _lib.load()
        self.mol = mol
        self._arrays = [np.ascontiguousarray(mol.Z, dtype=np.int32),
                        np.ascontiguousarray(mol.xyz, dtype=np.float64),
                        np.ascontiguousarray(mol.bf_atom, dtype=np.int32),
                        np.ascontiguousarray(mol.bf_lmn, dtype=np.int32),
                        np.ascontiguousarray(mol.bf_nprim, dtype=np.int32),
                        np.ascontiguousarray(mol.prim_alpha, dtype=np.float64),
                        np.ascontiguousarray(mol.prim_coef, dtype=np.float64)]
        Z, xyz, ba, bl, bn, pa, pc = self._arrays
        ip = ctypes.POINTER(ctypes.c_int)
        m = _lib.Molecule(mol.natoms, Z.ctypes.data_as(ip), _ptr(xyz))
        b = _lib.Basis(mol.nbf, ba.ctypes.data_as(ip), bl.ctypes.data_as(ip), bn.ctypes.data_as(ip), _ptr(pa), _ptr(pc))
        g = _lib.GridParams(radial_points, lebedev_order, lmax, device)
        h = ctypes.c_void_p()
        if cells is None:
            check(L.dftg_create(ctypes.byref(m), ctypes.byref(b), ctypes.byref(g), ctypes.byref(h)))
        else:
            check(L.dftg_create_cells(ctypes.byref(m), ctypes.byref(b), ctypes.byref(g), int(cells[0]), int(cells[1]),
                                      ctypes.byref(h)))
        self._h = h
        n = ctypes.c_size_t()
        check(L.dftg_grid_size(h, ctypes.byref(n)))
        self.grid_size = int(n.value)
        self.nbf = mol.nbf
        self.radial_points, self.lebedev_order, self.lmax = radial_points, lebedev_order, lmax
        self.set_precision(precision)

    # ------------------------------------------------------------ lifetime
    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.load().dftg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def set_precision(self, precision):
        code = {"fp64": _lib.DFTG_PREC_FP64, "mixed": _lib.DFTG_PREC_MIXED}[precision]
        check(_lib.load().dftg_set_precision(self._h, code))
        self.precision = precision

    MIX_BITS = {"density": 1, "lda": 2, "multipole": 4, "cross": 8, "contract": 16}

    def set_precision_mask(self, mask):
        """Run the steps whose bits are set (MIX_BITS) in the mixed form."""
        check(_lib.load().dftg_set_precision_mask(self._h, int(mask)))
        self.precision = "mixed" if mask else "fp64"

    def set_stream(self, stream_ptr):
        check(_lib.load().dftg_set_stream(self._h, ctypes.c_void_p(stream_ptr)))

    # ------------------------------------------------- reference interface
    def set_density(self, P):
        P = np.asfortranarray(P, dtype=np.float64)
        check(_lib.load().dftg_set_density(self._h, _ptr(P)))

    def correct_densities(self):
        c = ctypes.c_double()
        check(_lib.load().dftg_correct_densities(self._h, ctypes.byref(c)))
        return c.value

    def calculate_density(self):
        n = ctypes.c_double()
        check(_lib.load().dftg_calculate_density(self._h, ctypes.byref(n)))
        return n.value

    def calculate_hartree_potential(self):
        J = np.zeros((self.nbf, self.nbf), order="F")
        check(_lib.load().dftg_calculate_hartree_potential(self._h, _ptr(J)))
        return np.ascontiguousarray(J)

    def calculate_xc(self):
        XC = np.zeros((self.nbf, self.nbf), order="F")
        e = ctypes.c_double()
        check(_lib.load().dftg_calculate_xc(self._h, _ptr(XC), ctypes.byref(e)))
        return np.ascontiguousarray(XC), e.value

    def fock_build(self, P):
        """One grid Fock build at fixed P; returns J, XC, E_xc and the
        integrated (corrected) density."""
        P = np.asfortranarray(P, dtype=np.float64)
        J = np.zeros((self.nbf, self.nbf), order="F")
        XC = np.zeros((self.nbf, self.nbf), order="F")
        e, n = ctypes.c_double(), ctypes.c_double()
        check(_lib.load().dftg_fock_build(self._h, _ptr(P), _ptr(J), _ptr(XC), ctypes.byref(e), ctypes.byref(n)))
        return {"J": np.ascontiguousarray(J), "XC": np.ascontiguousarray(XC), "Exc": e.value, "nelec": n.value,
                "EJ": self.energies()["EJ"]}

    def backward(self, seed_exc=1.0, seed_ej=1.0):
        """Backward pass of the last fock_build (autograd-style vector-Jacobian
        product): for E = seed_exc E_xc + seed_ej E_J returns (dE/dP [nbf x nbf],
        dE/dR [natoms x 3] at fixed P).  The grid part of the nuclear forces
        is -dE/dR."""
        dP = np.zeros((self.nbf, self.nbf), order="F")
        dR = np.zeros((self.mol.natoms, 3))
        check(_lib.load().dftg_backward(self._h, float(seed_exc), float(seed_ej), _ptr(dP), _ptr(dR)))
        return np.ascontiguousarray(dP), dR

    def autotune(self, reps=10):
        """Time candidate launch shapes of the tensor-core kernels on the last
        built P and keep the fastest; returns the best ms per build."""
        ms = ctypes.c_double()
        check(_lib.load().dftg_autotune(self._h, int(reps), ctypes.byref(ms)))
        return ms.value

    @property
    def launch_shape(self):
        """(density CTAs, contraction CTAs, contraction stages); 0 = no such kernel."""
        v = (ctypes.c_int * 3)()
        check(_lib.load().dftg_get_launch_shape(self._h, v, 3))
        return tuple(v)

    @launch_shape.setter
    def launch_shape(self, shape):
        v = (ctypes.c_int * 3)(*[int(x) for x in shape])
        check(_lib.load().dftg_set_launch_shape(self._h, v, 3))

    def backward_profile(self, seed_exc=1.0, seed_ej=1.0):
        """Per-phase device times (ms) of one backward pass: {name: ms}."""
        ms = (ctypes.c_double * 32)()
        names = (ctypes.c_char_p * 32)()
        n = ctypes.c_int()
        check(_lib.load().dftg_backward_profile(self._h, float(seed_exc), float(seed_ej), ms, names, 32,
                                                ctypes.byref(n)))
        return {names[i].decode(): ms[i] for i in range(n.value)}

    def energies(self):
        """E_xc, E_J = 2 tr(P J) summed on the grid in FP64, integrated density
        of the last build."""
        e, j, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        check(_lib.load().dftg_get_energies(self._h, ctypes.byref(e), ctypes.byref(j), ctypes.byref(n)))
        return {"Exc": e.value, "EJ": j.value, "nelec": n.value}

    def _points(self, name, mult=1):
        out = np.empty(self.grid_size * mult)
        check(getattr(_lib.load(), name)(self._h, _ptr(out), out.size))
        return out

    def get_weights(self):
        return self._points("dftg_get_weights")

    def get_becke_weights(self):
        return self._points("dftg_get_becke_weights")

    def get_densities(self):
        return self._points("dftg_get_densities")

    def get_potential(self):
        return self._points("dftg_get_potential")

    def get_positions(self):
        return self._points("dftg_get_positions", 3).reshape(-1, 3)

    def get_amplitudes(self):
        """nbf x npts (the reference's orientation)."""
        out = np.empty(self.grid_size * self.nbf)
        check(_lib.load().dftg_get_amplitudes(self._h, _ptr(out), out.size))
        return out.reshape(self.grid_size, self.nbf).T

    def one_electron(self):
        n = self.nbf
        S, T, V = (np.zeros((n, n), order="F") for _ in range(3))
        check(_lib.load().dftg_one_electron(self._h, _ptr(S), _ptr(T), _ptr(V)))
        return np.ascontiguousarray(S), np.ascontiguousarray(T), np.ascontiguousarray(V)

    def eri_coulomb(self, P):
        """J_ij = sum_kl P_kl (ij|kl) from analytic two-electron integrals on the
        device (the reference's TWO_ELECTRON_INTEGRALS path, dft.cpp:452-477): an
        independent check of the grid J."""
        P = np.asfortranarray(P, dtype=np.float64)
        J = np.zeros((self.nbf, self.nbf), order="F")
        check(_lib.load().dftg_eri_coulomb(self._h, _ptr(P), _ptr(J)))
        return np.ascontiguousarray(J)

    def nuclear_repulsion(self):
        e = ctypes.c_double()
        check(_lib.load().dftg_nuclear_repulsion(self._h, ctypes.byref(e)))
        return e.value


class DFT:
    """Closed-shell LDA SCF driver with the reference's iteration
    (dft.cpp:84-142): F = H + 2J + XC, canonical orthogonalisation,
    P = C_occ C_occ^T, linear damping 0.5 after the first density."""

    def __init__(self, mol, radial_points=15, lebedev_order=7, lmax=8, precision="fp64", device=0):
        self.mol = mol
        self.molgrid = MolecularGrid(mol, radial_points, lebedev_order, lmax, precision, device)
        S, T, V = self.molgrid.one_electron()
        self.S, self.T, self.V = S, T, V
        self.H = T + V
        self.enuc = self.molgrid.nuclear_repulsion()
        lam, U = np.linalg.eigh(S)
        self.X = U @ np.diag(1.0 / np.sqrt(lam))
        n = mol.nbf
        self.J = np.zeros((n, n))
        self.XC = np.zeros((n, n))
        self.P = None
        self.exc = 0.0
        self.history = []
        # construct_matrices: first density from H, then J and the energy (dft.cpp:216-226)
        self._density_matrix()
        self.molgrid.set_density(self.P)
        self.molgrid.correct_densities()
        self.J = self.molgrid.calculate_hartree_potential()
        self.et = self._energy()

    def _density_matrix(self, alpha=0.5):
        F = self.H + 2.0 * self.J + self.XC
        _, Cp = np.linalg.eigh(self.X.T @ F @ self.X)
        C = self.X @ Cp
        nocc = self.mol.nelec // 2
        Pn = C[:, :nocc] @ C[:, :nocc].T
        self.P = Pn if self.P is None else (1.0 - alpha) * Pn + alpha * self.P

    def _energy(self):
        """dft.cpp:441-447.  In the mixed build the Hartree term is the grid sum
        of the library (the same 2 tr(P J), accumulated in FP64)."""
        self.e_one = 2.0 * np.trace(self.P @ self.H)
        if self.molgrid.precision == "mixed" and getattr(self, "e_j_grid", None) is not None:
            self.e_j = self.e_j_grid
        else:
            self.e_j = 2.0 * np.trace(self.P @ self.J)
        return self.e_one + self.e_j + self.enuc + self.exc

    def scf(self, tol=1e-4, max_iter=100, min_iter=3):
        old = self.et
        diff = 1.0
        it = 0
        while diff > tol or it < min_iter:
            it += 1
            self._density_matrix()
            r = self.molgrid.fock_build(self.P)
            self.J, self.XC, self.exc = r["J"], r["XC"], r["Exc"]
            self.e_j_grid = r["EJ"]
            self.et = self._energy()
            self.history.append({"iter": it, "E": self.et, "Exc": self.exc, "EJ": self.e_j, "nelec": r["nelec"]})
            diff = abs(self.et - old)
            old = self.et
            if it >= max_iter:
                break
        return self.et


class DeviceSCF:
    """The reference's DFT constructor + DFT::scf (dft.cpp:57-61, 84-142,
    160-227, 300-366) with every step on the GPU (dftg_scf_*): one-electron
    matrices, X, eigen-solves, damping, grid Fock builds and the energy.  run()
    is one CUDA graph launch for the whole loop."""

    def __init__(self, mol, radial_points=15, lebedev_order=7, lmax=8, precision="fp64", device=0,
                 alpha=0.5, tol=1e-4, min_iter=3, max_iter=100, nelec=0, refine_steps=0):
        self.mol = mol
        self.molgrid = MolecularGrid(mol, radial_points, lebedev_order, lmax, precision, device)
        self.nbf = mol.nbf
        prm = _lib.ScfParams(int(nelec), float(alpha), float(tol), int(min_iter), int(max_iter), int(refine_steps))
        check(_lib.load().dftg_scf_init(self.molgrid.handle, ctypes.byref(prm)))
        self.nocc = (nelec or int(np.sum(mol.Z))) // 2
        self.et = self.state()["E"]      # E_0 of the set-up (E_xc = 0)

    def state(self):
        """{E: last energy, iterations, dE: last |E_n - E_(n-1)|, running: the loop would continue}."""
        st = self._get(_lib.SCF_STATE, 4)
        return {"E": st[0], "iterations": int(st[1]), "dE": st[2], "running": bool(st[3])}

    def run(self):
        """Iterate to convergence; returns the final energy (DFT::scf)."""
        e, it = ctypes.c_double(), ctypes.c_int()
        check(_lib.load().dftg_scf_run(self.molgrid.handle, ctypes.byref(e), ctypes.byref(it)))
        self.et, self.iterations = e.value, it.value
        return e.value

    scf = run

    def step(self):
        """One iteration; returns (E, converged)."""
        e, conv = ctypes.c_double(), ctypes.c_int()
        check(_lib.load().dftg_scf_step(self.molgrid.handle, ctypes.byref(e), ctypes.byref(conv)))
        self.et = e.value
        return e.value, bool(conv.value)

    def _get(self, what, count, shape=None):
        out = np.zeros(max(count, 1))
        n = ctypes.c_size_t()
        check(_lib.load().dftg_scf_get(self.molgrid.handle, what, _ptr(out), out.size, ctypes.byref(n)))
        out = out[:n.value]
        return out if shape is None else out.reshape(shape, order="F")

    def matrix(self, name):
        """'P', 'J', 'XC', 'H' or 'X' (nbf x nbf)."""
        what = {"P": _lib.SCF_P, "J": _lib.SCF_J, "XC": _lib.SCF_XC, "H": _lib.SCF_H, "X": _lib.SCF_X}[name]
        return np.ascontiguousarray(self._get(what, self.nbf * self.nbf, (self.nbf, self.nbf)))

    @property
    def P(self):
        return self.matrix("P")

    def orbital_energies(self):
        return self._get(_lib.SCF_EPS, self.nbf)

    def occupied_coefficients(self):
        return self._get(_lib.SCF_COCC, self.nbf * self.nocc, (self.nbf, self.nocc))

    def history(self):
        """Per iteration of the last run: rows {E, 2tr(PH), E_J, E_xc, N, |dE|}."""
        h = self._get(_lib.SCF_HISTORY, _lib.SCF_HIST_W * _lib.SCF_MAX_ITER)
        return h.reshape(-1, _lib.SCF_HIST_W)

    def diagnostics(self):
        """{max |S'| across the occupied / virtual split, max |I - C'^T C'|,
        Jacobi sweeps, loop mode (1: conditional graph, 2: host-stepped)}."""
        d = self._get(_lib.SCF_DIAG, 4)
        return {"cross": d[0], "orth": d[1], "sweeps": int(d[2]), "mode": int(d[3])}

    def close(self):
        self.molgrid.close()


class PointGrid(MolecularGrid):
    """Explicit points and weights with functions about explicit centres (no
    atoms, cells or Hartree step): amplitudes, density, LDA point kernel and
    the XC contraction (dftg_create_points).  The MolecularGrid getters,
    precision and launch-shape calls apply."""

    def __init__(self, xyz, w, centres, bf_centre, bf_lmn, bf_nprim, prim_alpha, prim_coef, precision="fp64",
                 device=0):
        L = _lib.load()
        self.mol = None
        self._arrays = [np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3),
                        np.ascontiguousarray(w, dtype=np.float64),
                        np.ascontiguousarray(centres, dtype=np.float64).reshape(-1, 3),
                        np.ascontiguousarray(bf_centre, dtype=np.int32),
                        np.ascontiguousarray(bf_lmn, dtype=np.int32).reshape(-1, 3),
                        np.ascontiguousarray(bf_nprim, dtype=np.int32),
                        np.ascontiguousarray(prim_alpha, dtype=np.float64),
                        np.ascontiguousarray(prim_coef, dtype=np.float64)]
        X, W, C, bc, bl, bn, pa, pc = self._arrays
        ip = ctypes.POINTER(ctypes.c_int)
        zeros = np.zeros(len(C), dtype=np.int32)
        self._arrays.append(zeros)
        pts = _lib.Points(len(W), _ptr(X), _ptr(W))
        m = _lib.Molecule(len(C), zeros.ctypes.data_as(ip), _ptr(C))
        b = _lib.Basis(len(bc), bc.ctypes.data_as(ip), bl.ctypes.data_as(ip), bn.ctypes.data_as(ip), _ptr(pa),
                       _ptr(pc))
        h = ctypes.c_void_p()
        check(L.dftg_create_points(ctypes.byref(pts), ctypes.byref(m), ctypes.byref(b), int(device), ctypes.byref(h)))
        self._h = h
        self.grid_size = len(W)
        self.nbf = len(bc)
        self.set_precision(precision)

    def xc_build(self, P):
        """rho, LDA and XC at fixed P: {"XC", "Exc", "nelec"}."""
        P = np.asfortranarray(P, dtype=np.float64)
        XC = np.zeros((self.nbf, self.nbf), order="F")
        e, n = ctypes.c_double(), ctypes.c_double()
        check(_lib.load().dftg_xc_build(self._h, _ptr(P), _ptr(XC), ctypes.byref(e), ctypes.byref(n)))
        return {"XC": np.ascontiguousarray(XC), "Exc": e.value, "nelec": n.value}


class Batch:
    """Many MolecularGrid contexts built together (dftg_batch_*).  mode
    "persistent" (the default): every step of the mixed build is one persistent
    launch over all contexts, taking (context, block) items from a device queue;
    "graph": the per-build kernel sequences on one stream branch per context.
    Either form is captured into a CUDA graph and replayed.  Buffers are device
    tensors (torch), one set per context; build() returns nothing and does not
    synchronise (status() does, and reports expired bounded waits)."""

    MODES = {"persistent": 0, "graph": 1}

    def __init__(self, grids, mode="persistent"):
        self.grids = list(grids)
        n = len(self.grids)
        arr = (ctypes.c_void_p * n)(*[g.handle for g in self.grids])
        h = ctypes.c_void_p()
        check(_lib.load().dftg_batch_create(arr, n, ctypes.byref(h)))
        self._h = h.value
        self.set_mode(mode)

    def set_mode(self, mode):
        check(_lib.load().dftg_batch_set_mode(self._h, self.MODES[mode]))

    def persistent_active(self):
        """True when the last build ran as the persistent launches."""
        flag = ctypes.c_int()
        _lib.load().dftg_batch_get_mode(self._h, ctypes.byref(flag))
        return bool(flag.value)

    def status(self):
        """Synchronise the last batch; raises DftgError on an expired wait."""
        check(_lib.load().dftg_batch_status(self._h))

    def selftest_wait(self, limit_ms=20.0):
        """Return code of the persistent launches' bounded-wait self-test
        (DFTG_ERR_TIMEOUT expected)."""
        return _lib.load().dftg_batch_selftest_wait(self._h, float(limit_ms))

    def close(self):
        if getattr(self, "_h", None):
            _lib.load().dftg_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def autotune(self, reps=5):
        """Scale all contexts' CTA counts together (1, 1/2, 1/4, 1/8), keep the
        fastest for concurrent replay; returns ms per batch replay."""
        ms = ctypes.c_double()
        check(_lib.load().dftg_batch_autotune(self._h, int(reps), ctypes.byref(ms)))
        return ms.value

    def build(self, P_devs, J_devs=None, XC_devs=None, scal_devs=None, stream=None):
        n = len(self.grids)

        def ptrs(ts):
            if ts is None:
                return None
            return (ctypes.c_void_p * n)(*[t.data_ptr() if t is not None else None for t in ts])

        check(_lib.load().dftg_batch_fock_build_device(self._h, ptrs(P_devs), ptrs(J_devs), ptrs(XC_devs),
                                                       ptrs(scal_devs), stream))
