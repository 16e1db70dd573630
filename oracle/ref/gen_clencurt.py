#!/usr/bin/env python3
"""Generate the nested Clenshaw-Curtis tables that the reference's vendored
p-adaptive cubature (libs/libSGJC/pcubature.c:39, :104-108, :201-203, :382)
includes as ``clencurt.h``.  That header is absent from the reference tree
(listed in libs/libSGJC/Makefile.am:7), so the oracle build regenerates it
from the mathematics of the Clenshaw-Curtis rule:

* order m uses n = 2**(m+1) intervals on [-1, 1], nodes x_j = cos(j*pi/n);
* ``clencurt_x`` lists the positive non-centre nodes in nesting order: the
  node x=1 of order 0, then for each order m >= 1 the 2**(m-1) nodes that are
  new at that order (odd j);
* ``clencurt_w`` holds, for each order m at offset m + 2**m - 1, the centre
  weight followed by one weight per node of ``clencurt_x[0 : 2**m]`` (each such
  weight multiplies f(c + r x) + f(c - r x));
* weights are those of the rule on [-1, 1] (they sum to 2 when the symmetric
  pairs are counted twice), matching the trivial-rule weight of 2 used at
  pcubature.c:194.

Usage: gen_clencurt.py OUT.h [MAXORDER]
"""
import math
import sys


def cc_weights(n):
    """Clenshaw-Curtis weights w_j (j = 0..n) for nodes cos(j pi / n), n even."""
    import numpy as np
    j = np.arange(n + 1)[:, None]
    k = np.arange(1, n // 2 + 1)[None, :]
    b = np.where(2 * k == n, 1.0, 2.0)
    s = (b / (4.0 * k * k - 1.0) * np.cos(2.0 * k * j * math.pi / n)).sum(axis=1)
    c = np.where((j[:, 0] == 0) | (j[:, 0] == n), 1.0, 2.0)
    return list(c / n * (1.0 - s))


def main():
    out = sys.argv[1]
    mmax = int(sys.argv[2]) if len(sys.argv) > 2 else 11
    # cumulative node list as (level, odd index) -> x
    nodes = [(0, 0)]  # x = 1 at order 0 (j = 0)
    for m in range(1, mmax + 1):
        for jodd in range(1, 2 ** m, 2):
            nodes.append((m, jodd))
    xs = []
    for (lev, j) in nodes:
        n = 2 ** (lev + 1)
        xs.append(math.cos(j * math.pi / n))
    wtab = []
    for m in range(0, mmax + 1):
        n = 2 ** (m + 1)
        w = cc_weights(n)
        row = [w[n // 2]]
        for (lev, j) in nodes[: 2 ** m]:
            jj = j * 2 ** (m - lev)  # index of this node within the order-m rule
            row.append(w[jj])
        assert len(row) == 1 + 2 ** m
        wtab.extend(row)
    with open(out, "w") as f:
        f.write("/* generated by oracle/ref/gen_clencurt.py: nested Clenshaw-Curtis tables */\n")
        f.write("static const int clencurt_M = %d;\n" % mmax)
        f.write("static const double clencurt_x[%d] = {\n" % len(xs))
        f.write(",\n".join("%.17e" % x for x in xs))
        f.write("\n};\n")
        f.write("static const double clencurt_w[%d] = {\n" % len(wtab))
        f.write(",\n".join("%.17e" % x for x in wtab))
        f.write("\n};\n")


if __name__ == "__main__":
    main()
