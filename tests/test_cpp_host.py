"""The C++ host mirror (include/dftg.hpp): compiles against the C ABI on the
CPU; on the GPU its SCF reproduces the Python driver's energies."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from dftcxx_gb300.molecule import Molecule, h2o

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _compile(tmp):
    from dftcxx_gb300 import build
    build.build()
    exe = os.path.join(tmp, "host_scf")
    libdir = os.path.join(ROOT, "dftcxx_gb300")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "host_scf.cpp"), "-o", exe, "-L", libdir, "-ldftg",
           "-Wl,-rpath," + libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "warning" not in r.stderr, r.stderr
    return exe


def _write_molecule(path, mol):
    with open(path, "w") as f:
        f.write("%d %d %d\n" % (mol.natoms, mol.nbf, len(mol.prim_alpha)))
        for z, (x, y, w) in zip(mol.Z, mol.xyz):
            f.write("%d %.17g %.17g %.17g\n" % (z, x, y, w))
        for a, lmn, n in zip(mol.bf_atom, mol.bf_lmn, mol.bf_nprim):
            f.write("%d %d %d %d %d\n" % (a, lmn[0], lmn[1], lmn[2], n))
        for al, c in zip(mol.prim_alpha, mol.prim_coef):
            f.write("%.17g %.17g\n" % (al, c))


@pytest.mark.skipif(shutil.which("g++") is None, reason="no C++ compiler")
def test_cpp_mirror_compiles(tmp_path):
    exe = _compile(str(tmp_path))
    assert os.path.exists(exe)


@pytest.mark.skipif(shutil.which("g++") is None, reason="no C++ compiler")
def test_host_jacobi_eigensolver(tmp_path):
    """jacobi_eigh of dftg.hpp (the SCF's eigen-solver) against numpy on a
    random symmetric matrix of benzene / 6-31G size and an S-like matrix."""
    exe = str(tmp_path / "jacobi_check")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "jacobi_check.cpp"), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    rng = np.random.default_rng(5)
    for n in (7, 66):
        B = rng.normal(size=(n, n))
        A = B @ B.T / n + np.eye(n) * 1e-3
        inp = "%d\n" % n + "\n".join("%.17g" % x for x in A.ravel(order="F"))
        out = subprocess.run([exe], input=inp, capture_output=True, text=True, check=True).stdout.split()
        vals = np.array([float(x) for x in out])
        w, V = vals[:n], vals[n:].reshape(n, n, order="F")
        wr = np.linalg.eigvalsh(A)
        assert np.abs(w - wr).max() < 1e-12 * np.abs(wr).max()
        assert np.abs(A @ V - V * w).max() < 1e-11 * np.abs(wr).max()
        assert np.abs(V.T @ V - np.eye(n)).max() < 1e-12


@pytest.mark.gpu
def test_cpp_mirror_scf_matches_python(gpu_lib, tmp_path):
    from dftcxx_gb300.grid import DFT
    exe = _compile(str(tmp_path))
    Z, xyz = h2o()
    mol = Molecule(Z, xyz, "sto3g")
    mf = str(tmp_path / "h2o.txt")
    _write_molecule(mf, mol)
    d = DFT(mol, 32, 7, 8, precision="fp64")
    e_py = d.scf(tol=1e-8)
    for mode in ([], ["device"]):
        r = subprocess.run([exe, mf, "32", "7", "8", "fp64", "1e-8"] + mode, capture_output=True, text=True,
                           timeout=300)
        assert r.returncode == 0, r.stderr
        last = [l for l in r.stdout.splitlines() if l.startswith("E ")][-1].split()
        e_cpp, iters = float(last[1]), int(last[3])
        its = [float(l.split()[1]) for l in r.stdout.splitlines() if l.startswith("IT ")]
        assert iters == len(d.history) == len(its), mode
        assert abs(e_cpp - e_py) < 1e-9, mode
        assert max(abs(a - h["E"]) for a, h in zip(its, d.history)) < 1e-9, mode
