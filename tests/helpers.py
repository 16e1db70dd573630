"""Shared helpers for the tests: build gbem / oracle geometries from fixtures."""
import numpy as np


def fixture_surfaces(d):
    """(list of gbem surface dicts, oracle args) from a ref_*.npz fixture."""
    from gbem.api import Material
    n = int(d["objects"])
    gs, regs, pec, eps, mu = [], [], [], [1.0], [1.0]
    for i in range(n):
        V = d["V%d" % i] + d["disp%d" % i]
        P = d["P%d" % i]
        mat = str(d["mat%d" % i])
        if mat == "PEC":
            gs.append({"V": V, "P": P, "material": None})
            regs.append((0, -1)); pec.append(True)
        else:
            m = Material.parse(mat)
            gs.append({"V": V, "P": P, "material": m})
            eps.append(m.eps); mu.append(m.mu)
            regs.append((0, len(eps) - 1)); pec.append(False)
    return gs, (regs, pec, eps, mu)


def omega_of(d):
    return d["omega"][0] + 1j * d["omega"][1]


def relerr(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())
