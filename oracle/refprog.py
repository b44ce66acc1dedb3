"""Driver of the reference program's own code (oracle/_ref/ref_dump*).

TEST INFRASTRUCTURE: used by tests/golden/make_goldens.py to record what the
reference computes, and by the CPU-baseline leg of bench.py where the binary
exists.  ref_dump links the reference's unmodified translation units with the
Eigen/Boost API subset of oracle/shim (oracle/Makefile); ref_dump302 is the
same program with the 302-point Lebedev rule added to its quadrature table.

The reference reads its basis set from ../basis/<name>.dat relative to the
working directory (molecule.cpp:147-152), so every run gets a scratch folder
with a ``basis`` folder and a working folder next to it.  The basis file is
written in the reference's format (molecule.cpp:135-238: ``Z ncgf``, then
``TYPE nprim``, then tab-led ``exponent coefficient`` lines) from the
repository's JSON copy of the same published data, whose numbers are
hash-checked against the reference's files (tests/test_oracle.py); every
number is written with repr, so the reference parses the same doubles.
"""
import json
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
BASIS_DIR = os.path.join(os.path.dirname(HERE), "dftcxx_gb300", "basis")
SYMBOL = {1: "H", 2: "He", 3: "Li", 4: "Be", 5: "B", 6: "C", 7: "N", 8: "O", 9: "F", 10: "Ne",
          11: "Na", 12: "Mg", 13: "Al", 14: "Si", 15: "P", 16: "S", 17: "Cl", 18: "Ar"}


def build(ref_root):
    """Compile ref_dump and ref_dump302 from the reference sources under ref_root/src."""
    src = os.path.join(ref_root, "src")
    subprocess.check_call(["make", "-s", "-j8", "-C", HERE, "refdump", "refdump302", "REFSRC=" + src])


def binary(lebedev_order):
    return os.path.join(REF_DIR, "ref_dump302" if lebedev_order == 11 else "ref_dump")


def available(lebedev_order=7):
    return os.path.exists(binary(lebedev_order))


def input_text(name, basis, Z, xyz, nrad, lebedev_order, lmax):
    """A reference input file (settings.cpp:39-70, molecule.cpp:61-128) in bohr.
    hartree_evaluation is given a value other than the two the reference names:
    settings.cpp:104-107 leaves the method unset for "becke_grid" and the
    default, and sets the Becke grid for any other string."""
    lines = ["name = %s" % name, "basis = %s" % basis, "units = bohr", "hartree_evaluation = becke",
             "radial_points = %d" % nrad, "lebedev_order = %d" % lebedev_order, "lmax = %d" % lmax, "",
             "system:", "%d" % len(Z)]
    for z, (x, y, w) in zip(Z, xyz):
        lines.append("%s %.17g %.17g %.17g" % (SYMBOL[int(z)], x, y, w))
    return "\n".join(lines) + "\n"


def basis_dat(name):
    """The basis set `name` in the reference's .dat layout."""
    with open(os.path.join(BASIS_DIR, name + ".json")) as f:
        data = json.load(f)
    lines = []
    for z in sorted(data, key=int):
        lines.append("%s\t%d" % (z, len(data[z])))
        for kind, prims in data[z]:
            lines.append("%s\t%d" % (kind, len(prims)))
            lines += ["\t%r\t%r" % (float(a), float(c)) for a, c in prims]
    return "\n".join(lines) + "\n"


def _run(basis, text, args, lebedev_order, threads=None, timeout=3600):
    exe = binary(lebedev_order)
    if not os.path.exists(exe):
        raise RuntimeError("%s is not built (oracle/Makefile refdump / refdump302)" % exe)
    with tempfile.TemporaryDirectory() as tmp:
        os.makedirs(os.path.join(tmp, "basis"))
        with open(os.path.join(tmp, "basis", basis + ".dat"), "w") as f:
            f.write(basis_dat(basis))
        work = os.path.join(tmp, "run")
        os.makedirs(work)
        inp = os.path.join(work, "mol.in")
        with open(inp, "w") as f:
            f.write(text)
        out = os.path.join(tmp, "out")
        env = dict(os.environ)
        if threads:
            env["OMP_NUM_THREADS"] = str(threads)
        full = [exe, inp, out] + [a(tmp) if callable(a) else a for a in args]
        r = subprocess.run(full, cwd=work, env=env, capture_output=True, text=True, timeout=timeout)
        if r.returncode != 0:
            raise RuntimeError("ref_dump failed (%d): %s" % (r.returncode, r.stderr[-2000:]))
        res = {os.path.splitext(f)[0]: np.load(os.path.join(out, f)) for f in os.listdir(out)}
        res["log"] = r.stdout
        return res


def fock_build(mol, nrad, lebedev_order, lmax, P, amp=False, threads=None):
    """The reference's build at a fixed half density matrix P (nbf x nbf):
    weights, becke, rho (corrected), potential, positions, J, XC, P, S, T,
    Vnuc, H; scalars = [E_xc, E_J = 2tr(PJ), 2tr(PH), E_nuc, E_tot, integral
    of w rho before and after the correction]; timings_ms = [set_density,
    correct_densities, Hartree (J), XC, energy, constructor]."""
    text = input_text(mol.name or "molecule", mol.basis_name, mol.Z, mol.xyz, nrad, lebedev_order, lmax)
    Pf = np.asfortranarray(np.asarray(P, dtype=np.float64))

    def pfile(tmp):
        path = os.path.join(tmp, "P.bin")
        Pf.ravel(order="F").tofile(path)
        return path

    args = ["build", pfile] + (["amp"] if amp else [])
    return _run(mol.basis_name, text, args, lebedev_order, threads)


def scf(mol, nrad, lebedev_order, lmax, max_iter=100, tol=1e-8, threads=None):
    """The reference's SCF loop from its core-Hamiltonian guess: history rows
    [E_tot, 2tr(PH), 2tr(PJ), E_xc, N] per iteration, final P, J, XC."""
    text = input_text(mol.name or "molecule", mol.basis_name, mol.Z, mol.xyz, nrad, lebedev_order, lmax)
    return _run(mol.basis_name, text, ["scf", str(int(max_iter)), repr(float(tol))], lebedev_order, threads)
