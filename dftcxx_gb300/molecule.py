"""Molecule, basis set and settings input for the grid Fock build.

Mirrors the input side of DFTCXX: ``Settings`` (settings.cpp:29-187),
``Molecule::read_molecule_from_file`` (molecule.cpp:61-128) and
``Molecule::set_basis_set`` (molecule.cpp:135-238).  Basis functions are
ordered exactly as the reference orders them: by element in basis-file order
(increasing Z), then by atom in input order, then shell by shell with P shells
expanded to (x, y, z) and D shells to (xx, xy, xz, yy, yz, zz).
"""
import json
import math
import os
import re

import numpy as np

ANGSTROM_TO_BOHR = 1.889725989          # molecule.cpp:66
ELEMENTS = ["H", "He", "Li", "Be", "B", "C", "N", "O", "F", "Ne", "Na",
            "Mg", "Al", "Si", "P", "S", "Cl", "Ar"]   # molecule.cpp:277-278

# (l, m, n) per shell type, cgf.h:208-221 / cgf.cpp:185-232
SHELL_LMN = {
    "S": [(0, 0, 0)],
    "P": [(1, 0, 0), (0, 1, 0), (0, 0, 1)],
    "D": [(2, 0, 0), (1, 1, 0), (1, 0, 1), (0, 2, 0), (0, 1, 1), (0, 0, 2)],
}

# Lebedev orders (settings.h:64-78) plus the 302-point extension at index 11
LEBEDEV_NPTS = [6, 14, 26, 38, 50, 74, 86, 110, 146, 170, 194, 302]
LEBEDEV_302 = 11

# grid presets (settings.cpp:158-187): (radial points, lebedev order, lmax)
GRID_PRESETS = {
    "coarse": (10, 4, 5),
    "medium": (15, 7, 8),
    "fine": (20, 8, 10),
    "ultrafine": (30, 10, 11),
}

BASIS_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "basis")


def _split(line):
    # boost::split(..., is_any_of(" \t"), token_compress_on): a leading
    # separator yields an empty first token.
    return re.split(r"[ \t]+", line)


def parse_basis_dat(text):
    """Parse a DFTCXX basis file into ``{Z: [[type, [[alpha, coef], ...]], ...]}``."""
    lines = text.splitlines()
    out = {}
    i = 0
    while i < len(lines):
        line = lines[i]
        i += 1
        if not line or line[0] == "#":
            continue
        p = _split(line)
        z, ncgf = int(p[0]), int(p[1])
        shells = []
        for _ in range(ncgf):
            p = _split(lines[i])
            i += 1
            typ, nprim = p[0][0], int(p[1])
            prims = []
            for _ in range(nprim):
                q = _split(lines[i])
                i += 1
                prims.append([float(q[1]), float(q[2])])
            shells.append([typ, prims])
        out[z] = shells
    return out


_BASIS_CACHE = {}


def load_basis(name):
    """Load a basis set shipped with the package (sto3g, sto6g, p321, p631)
    or a DFTCXX ``.dat`` file given by path."""
    if name in _BASIS_CACHE:
        return _BASIS_CACHE[name]
    if os.path.exists(name):
        with open(name) as f:
            data = parse_basis_dat(f.read())
    else:
        with open(os.path.join(BASIS_DIR, name + ".json")) as f:
            data = {int(k): v for k, v in json.load(f).items()}
    _BASIS_CACHE[name] = data
    return data


class Molecule:
    """Atoms (bohr) plus contracted Gaussian basis functions.

    Flattened basis description (the layout of ``dftg_basis`` in dftg.h):
    ``bf_atom[nbf]``, ``bf_lmn[nbf,3]``, ``bf_nprim[nbf]``, and the primitive
    exponents/coefficients concatenated in basis-function order.
    """

    def __init__(self, Z, xyz, basis="sto3g", name=""):
        self.name = name
        self.Z = np.asarray(Z, dtype=np.int32)
        self.xyz = np.ascontiguousarray(np.asarray(xyz, dtype=np.float64).reshape(-1, 3))
        self.basis_name = basis
        self._build_basis(load_basis(basis))

    def _build_basis(self, data):
        bf_atom, bf_lmn, bf_nprim, alpha, coef = [], [], [], [], []
        highest = int(self.Z.max())
        for z in sorted(data):
            if z > highest:
                break
            if z not in self.Z:
                continue
            for a in range(len(self.Z)):
                if self.Z[a] != z:
                    continue
                for typ, prims in data[z]:
                    for lmn in SHELL_LMN[typ]:
                        bf_atom.append(a)
                        bf_lmn.append(lmn)
                        bf_nprim.append(len(prims))
                        alpha.extend(p[0] for p in prims)
                        coef.extend(p[1] for p in prims)
        missing = set(int(z) for z in self.Z) - set(int(z) for z in data)
        if missing:
            raise ValueError("basis %s has no data for Z=%s" % (self.basis_name, sorted(missing)))
        self.bf_atom = np.asarray(bf_atom, dtype=np.int32)
        self.bf_lmn = np.ascontiguousarray(np.asarray(bf_lmn, dtype=np.int32).reshape(-1, 3))
        self.bf_nprim = np.asarray(bf_nprim, dtype=np.int32)
        self.prim_alpha = np.asarray(alpha, dtype=np.float64)
        self.prim_coef = np.asarray(coef, dtype=np.float64)

    @property
    def natoms(self):
        return int(self.Z.shape[0])

    @property
    def nbf(self):
        return int(self.bf_atom.shape[0])

    @property
    def nelec(self):
        return int(self.Z.sum())

    def nuclear_repulsion(self):
        e = 0.0
        for i in range(self.natoms):
            for j in range(i + 1, self.natoms):
                e += self.Z[i] * self.Z[j] / np.linalg.norm(self.xyz[i] - self.xyz[j])
        return float(e)

    def displaced(self, dxyz):
        m = Molecule(self.Z, self.xyz + np.asarray(dxyz).reshape(-1, 3), self.basis_name, self.name)
        return m


class Settings:
    """Key/value header of a DFTCXX input file (settings.cpp:39-70) with the
    grid defaults of settings.cpp:91-151.  ``hartree_evaluation`` is parsed
    with a defined result for every value (the reference leaves it
    uninitialised for the default, settings.cpp:104-107)."""

    def __init__(self, values=None):
        self.values = dict(values or {})
        preset = GRID_PRESETS.get(self.values.get("grid", "medium"), GRID_PRESETS["medium"])
        self.radial_points, self.lebedev_order, self.lmax = preset
        for key in ("radial_points", "lebedev_order", "lmax"):
            if key in self.values:
                try:
                    setattr(self, key, int(self.values[key]))
                except ValueError:
                    pass
        he = self.values.get("hartree_evaluation", "becke_grid")
        self.hartree_evaluation = "two_electron_integrals" if he == "two_electron_integrals" else "becke_grid"


def read_input(path, basis_dir=None):
    """Read a DFTCXX ``.in`` file; returns ``(Settings, Molecule)``."""
    with open(path) as f:
        lines = f.read().splitlines()
    values = {}
    k = 0
    while k < len(lines):
        line = lines[k]
        k += 1
        pieces = [p for p in re.split(r"=+", line)]
        if len(pieces) == 2:
            values[pieces[0].strip()] = pieces[1].strip()
        if re.match(r"^system:\s*$", line):
            break
    settings = Settings(values)
    nat = int(lines[k].strip())
    Z, xyz = [], []
    for i in range(nat):
        p = _split(lines[k + 1 + i])
        Z.append(ELEMENTS.index(p[0]) + 1)
        v = [float(p[1]), float(p[2]), float(p[3])]
        if values.get("units") == "angstrom":
            v = [c * ANGSTROM_TO_BOHR for c in v]
        xyz.append(v)
    basis = values["basis"]
    if basis_dir is not None:
        basis = os.path.join(basis_dir, basis + ".dat")
    return settings, Molecule(Z, xyz, basis, values.get("name", ""))


# ------------------------------------------------------------------ geometries

def h2o():
    """H2O: O at the origin, H at (+-1.430, 1.107, 0) bohr."""
    return [8, 1, 1], [[0.0, 0.0, 0.0], [1.430, 1.107, 0.0], [-1.430, 1.107, 0.0]]


def benzene():
    """Benzene D6h: C on a 2.640 bohr ring (C-C 2.640), H at 4.680 bohr, z = 0."""
    Z, xyz = [], []
    for k in range(6):
        t = k * math.pi / 3.0
        Z.append(6)
        xyz.append([2.640 * math.cos(t), 2.640 * math.sin(t), 0.0])
    for k in range(6):
        t = k * math.pi / 3.0
        Z.append(1)
        xyz.append([4.680 * math.cos(t), 4.680 * math.sin(t), 0.0])
    return Z, xyz


def alkane(n, rcc=2.910, rch=2.060):
    """Staggered all-trans CnH2n+2 (n >= 2) with tetrahedral angles (bohr).

    Carbons zig-zag in the xy plane; each CH2 carries two H out of the plane
    along the bisector away from its carbon neighbours; each chain end carries
    one in-plane H where the next carbon would sit."""
    tet = math.acos(-1.0 / 3.0)
    half = tet / 2.0
    dx, dy = rcc * math.sin(half), rcc * math.cos(half)
    C = [[i * dx, (dy if i % 2 else 0.0), 0.0] for i in range(n)]
    Z, xyz = [6] * n, [list(c) for c in C]
    for i in range(n):
        up = -1.0 if i % 2 == 0 else 1.0
        for s in (-1.0, 1.0):
            v = [0.0, up * math.cos(half) * rch, s * math.sin(half) * rch]
            Z.append(1)
            xyz.append([C[i][k] + v[k] for k in range(3)])
    for end, sgn in ((0, -1.0), (n - 1, 1.0)):
        up = -1.0 if end % 2 == 0 else 1.0
        v = [sgn * math.sin(half) * rch, -up * math.cos(half) * rch, 0.0]
        Z.append(1)
        xyz.append([C[end][k] + v[k] for k in range(3)])
    return Z, xyz


def small_molecule(name):
    """Equilibrium-like geometries (bohr) for the batched workload."""
    if name == "H2":
        return [1, 1], [[0, 0, -0.7], [0, 0, 0.7]]
    if name == "LiH":
        return [3, 1], [[0, 0, 0], [0, 0, 3.015]]
    if name == "H2O":
        return h2o()
    if name == "NH3":
        r, th = 1.913, math.radians(106.7)
        h = r * math.cos(math.asin(math.sin(th / 2) * 2 / math.sqrt(3)))
        rho = math.sqrt(r * r - h * h)
        xyz = [[0, 0, 0]] + [[rho * math.cos(2 * math.pi * k / 3), rho * math.sin(2 * math.pi * k / 3), -h]
                             for k in range(3)]
        return [7, 1, 1, 1], xyz
    if name == "CH4":
        d = 2.052 / math.sqrt(3.0)
        return [6, 1, 1, 1, 1], [[0, 0, 0], [d, d, d], [-d, -d, d], [-d, d, -d], [d, -d, -d]]
    if name == "N2":
        return [7, 7], [[0, 0, -1.037], [0, 0, 1.037]]
    if name == "CO":
        return [6, 8], [[0, 0, -1.066], [0, 0, 1.066]]
    if name == "C2H6":
        return alkane(2)
    if name == "C6H6":
        return benzene()
    raise KeyError(name)


def synthetic_contraction(npts=2_000_000, nbf=512, nocc=128, seed=20261203, box=20.0):
    """Seeded synthetic contraction workload: points uniform in a cube, weights
    log-uniform in [1e-4, 1], single-primitive Cartesian s/p/d functions with
    log-uniform exponents in [0.1, 50], density P = C C^T with C ~ N(0, 0.1)."""
    rng = np.random.default_rng(seed)
    pts = rng.uniform(0.0, box, size=(npts, 3))
    w = np.exp(rng.uniform(math.log(1e-4), 0.0, size=npts))
    types = rng.integers(0, 10, size=nbf)
    all_lmn = SHELL_LMN["S"] + SHELL_LMN["P"] + SHELL_LMN["D"]
    lmn = np.asarray([all_lmn[t] for t in types], dtype=np.int32)
    alpha = np.exp(rng.uniform(math.log(0.1), math.log(50.0), size=nbf))
    centres = rng.uniform(0.0, box, size=(nbf, 3))
    C = rng.normal(0.0, 0.1, size=(nbf, nocc))
    P = C @ C.T
    return pts, w, lmn, alpha, centres, P
