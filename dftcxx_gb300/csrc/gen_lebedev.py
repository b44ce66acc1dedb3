"""Generate ``lebedev_data.h``: Lebedev-Laikov angular quadrature rules.

The rules come from ``scipy.integrate.lebedev_rule`` (the published
Lebedev-Laikov points and weights).  Each rule is rewritten in the layout the
DFTCXX grid code expects (quadrature.h:47-968 of the reference):

* rows of ``{x, y, z, w}`` with ``w`` normalised to sum to 1 (not 4*pi);
* every value rounded to 12 decimals;
* points grouped by octahedral orbit in the order SciPy lists the orbits, and
  inside each orbit expanded from the orbit's first point in the classic
  generator order (sign patterns ``+++ -++ +-+ --+ ++- -+- +-- ---`` over the
  coordinate permutations listed in ``_ORBIT_PERMS``).

Orders 0..10 are the reference's enum (settings.h:64-78: 6 .. 194 points).
Order 11 (302 points, algebraic degree 29) is an extension that the reference
does not ship.  Run ``python gen_lebedev.py`` to rewrite the header.
"""
import os
import numpy as np

DEGREES = [3, 5, 7, 9, 11, 13, 15, 17, 19, 21, 23, 29]
NPOINTS = [6, 14, 26, 38, 50, 74, 86, 110, 146, 170, 194, 302]

_SIGNS = [(1, 1, 1), (-1, 1, 1), (1, -1, 1), (-1, -1, 1),
          (1, 1, -1), (-1, 1, -1), (1, -1, -1), (-1, -1, -1)]


def _dedup(pts):
    out = []
    for p in pts:
        if not any(all(abs(p[i] - q[i]) < 1e-14 for i in range(3)) for q in out):
            out.append(p)
    return out


def _signed(v):
    return _dedup([(s[0] * v[0], s[1] * v[1], s[2] * v[2]) for s in _SIGNS])


def _expand(first):
    """Expand an orbit from its first point in generator order."""
    x, y, z = first
    ax = [abs(x), abs(y), abs(z)]
    nz = sum(1 for v in ax if v > 1e-12)
    if nz == 1:                       # (a,0,0): 6 points
        a = max(ax)
        return [(a, 0, 0), (-a, 0, 0), (0, a, 0), (0, -a, 0), (0, 0, a), (0, 0, -a)]
    if nz == 2 and abs(sorted(ax)[1] - sorted(ax)[2]) < 1e-9:   # (0,a,a): 12
        a = max(ax)
        return (_signed((0, a, a)) + _signed((a, 0, a)) + _signed((a, a, 0)))
    if nz == 3 and abs(ax[0] - ax[1]) < 1e-9 and abs(ax[1] - ax[2]) < 1e-9:  # (a,a,a): 8
        return _signed((ax[0], ax[0], ax[0]))
    if nz == 3 and abs(ax[0] - ax[1]) < 1e-9:                # (a,a,b): 24
        a, b = ax[0], ax[2]
        return _signed((a, a, b)) + _signed((a, b, a)) + _signed((b, a, a))
    if nz == 2:                                                # (a,b,0): 24
        a, b = ax[0], ax[1]
        out = []
        for v in [(a, b, 0), (b, a, 0), (a, 0, b), (b, 0, a), (0, a, b), (0, b, a)]:
            out += _signed(v)
        return out
    a, b, c = ax                                               # (a,b,c): 48
    out = []
    for v in [(a, b, c), (a, c, b), (b, a, c), (b, c, a), (c, a, b), (c, b, a)]:
        out += _signed(v)
    return out


def lebedev_rows(degree):
    from scipy.integrate import lebedev_rule
    xyz, w = lebedev_rule(degree)
    w = w / (4.0 * np.pi)
    n = w.shape[0]
    rows = []
    i = 0
    while i < n:
        first = (xyz[0, i], xyz[1, i], xyz[2, i])
        orbit = _expand(first)
        for p in orbit:
            rows.append((p[0], p[1], p[2], w[i]))
        i += len(orbit)
    assert len(rows) == n, (degree, len(rows), n)
    # check the orbit expansion reproduces SciPy's point set
    got = np.array(rows)
    ref = np.vstack([xyz, w[None]]).T
    d = np.abs(got[:, None, :] - ref[None, :, :]).max(-1).min(1)
    assert d.max() < 1e-13, (degree, d.max())
    return np.round(got, 12)


def main():
    here = os.path.dirname(os.path.abspath(__file__))
    lines = ["// Generated by gen_lebedev.py from scipy.integrate.lebedev_rule.",
             "// Lebedev-Laikov rules, rows {x, y, z, w}, weights summing to 1,",
             "// 12-decimal values, orbit-ordered.  Do not edit by hand.",
             "#pragma once",
             "#define DFTG_NUM_LEBEDEV_ORDERS %d" % len(NPOINTS),
             "static const int dftg_lebedev_npts[%d] = {%s};" % (
                 len(NPOINTS), ", ".join(str(n) for n in NPOINTS)),
             "static const int dftg_lebedev_offset[%d] = {%s};" % (
                 len(NPOINTS), ", ".join(str(sum(NPOINTS[:i])) for i in range(len(NPOINTS)))),
             "#define DFTG_LEBEDEV_TOTAL %d" % sum(NPOINTS),
             "static const double dftg_lebedev_table[%d][4] = {" % sum(NPOINTS)]
    for deg, npt in zip(DEGREES, NPOINTS):
        rows = lebedev_rows(deg)
        lines.append("    // %d points (degree %d)" % (npt, deg))
        for r in rows:
            lines.append("    {%s}," % ", ".join("%.12f" % (v + 0.0) for v in r))
    lines.append("};")
    with open(os.path.join(here, "lebedev_data.h"), "w") as f:
        f.write("\n".join(lines) + "\n")


if __name__ == "__main__":
    main()
