"""Write a quadrature.h with the reference's class layout and a 302-point rule.

TEST INFRASTRUCTURE.  The reference ships Lebedev orders 0-10 (6..194 points,
quadrature.h:47-968) and no 302-point rule, so its own code cannot build the
benzene / 6-31G / 75 x 302 grid.  This script writes, into a build folder
under oracle/_ref/, a header that declares the same class (Quadrature, its
order enum, num_lebedev_points, num_lebedev_coefficients, lebedev_coefficients)
with a twelfth order, LEBEDEV_302.  The rows come from the repository's
generated table (dftcxx_gb300/csrc/lebedev_data.h), whose first 914 rows are
byte-identical to the reference's table (tests/test_oracle.py checks that).
oracle/Makefile compiles the reference's translation units against it, with
every other reference file used from where it lies.

Usage: python oracle/gen_ref_quadrature.py OUT_HEADER
"""
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
TABLE = os.path.join(os.path.dirname(HERE), "dftcxx_gb300", "csrc", "lebedev_data.h")


def rows():
    txt = open(TABLE).read()
    npts = [int(x) for x in re.search(r"dftg_lebedev_npts\[\d+\] = \{([^}]*)\}", txt).group(1).split(",")]
    body = txt[txt.index("dftg_lebedev_table"):]
    vals = re.findall(r"\{(-?\d+\.\d+), (-?\d+\.\d+), (-?\d+\.\d+), (-?\d+\.\d+)\}", body)
    assert len(vals) == sum(npts), (len(vals), sum(npts))
    return npts, vals


def main(out):
    npts, vals = rows()
    names = ["LEBEDEV_%d" % n for n in npts]
    lines = [
        "// Generated by oracle/gen_ref_quadrature.py (test infrastructure): the",
        "// reference's Quadrature class with a 302-point Lebedev order appended.",
        "#ifndef _QUADRATURE_H",
        "#define _QUADRATURE_H",
        "",
        "#include <iostream>",
        "",
        "class Quadrature {",
        "public:",
        "    enum {",
    ]
    lines += ["        %s," % n for n in names]
    lines += ["", "        NUM_LEBEDEV_POINTS", "    };", ""]
    lines.append("    static constexpr unsigned int num_lebedev_points[%d] = {%s};"
                 % (len(npts), ", ".join(str(n) for n in npts)))
    lines.append("    static constexpr unsigned int num_lebedev_coefficients = %d;" % sum(npts))
    lines.append("    static constexpr double lebedev_coefficients[num_lebedev_coefficients][4] = {")
    lines += ["        {%s, %s, %s, %s}," % v for v in vals]
    lines += ["    };", "};", "", "#endif //_QUADRATURE_H", ""]
    os.makedirs(os.path.dirname(os.path.abspath(out)), exist_ok=True)
    with open(out, "w") as f:
        f.write("\n".join(lines))


if __name__ == "__main__":
    main(sys.argv[1])
