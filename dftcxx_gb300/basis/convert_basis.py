"""Convert DFTCXX basis-set data files (``basis/<name>.dat``) to JSON.

The numbers are the published STO-3G, STO-6G, 3-21G and 6-31G parameters
(Basis Set Exchange).  They are read from the reference's data files so the
inputs of this build are bit-identical to the reference's.  The file format
(molecule.cpp:135-238): ``Z ncgf`` then per shell ``TYPE nprim`` then ``nprim``
lines ``<blank-or-index> exponent coefficient``; lines starting with ``#`` are
comments.

Usage: python convert_basis.py <dir with sto3g.dat ...>
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from dftcxx_gb300.molecule import parse_basis_dat  # noqa: E402


def main(src):
    for name in ("sto3g", "sto6g", "p321", "p631"):
        path = os.path.join(src, name + ".dat")
        with open(path) as f:
            data = parse_basis_dat(f.read())
        out = {str(z): shells for z, shells in sorted(data.items())}
        with open(os.path.join(HERE, name + ".json"), "w") as f:
            json.dump(out, f, indent=0, separators=(",", ":"))
            f.write("\n")


if __name__ == "__main__":
    main(sys.argv[1])
