#!/usr/bin/env python3
"""Write gbem_fippi_cache_s1.bin: this library's FIPPI cache file (the
reference's format) for the dielectric s=1 sphere of ref_fippi_cache_s1_mesh.npz
at kR = 2.  Needs a GPU (the static table is computed there); the CPU test
tests/test_fippi_cache_cpu.py then has the reference itself read it.

  python tests/golden/make_gbem_cache.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(HERE)), "scuff-em_gb300"))
from gbem import RWGGeometry  # noqa: E402
from gbem.api import ClearCache, Material, StoreCache  # noqa: E402


def main(out=os.path.join(HERE, "gbem_fippi_cache_s1.bin")):
    ClearCache()
    m = np.load(os.path.join(HERE, "ref_fippi_cache_s1_mesh.npz"))
    G = RWGGeometry([{"V": m["V"], "P": m["P"], "material": Material(2.25 + 0.01j)}])
    G.AssembleBEMMatrix(2.0)
    StoreCache(out)
    print(out, os.path.getsize(out))


if __name__ == "__main__":
    main(*sys.argv[1:])
