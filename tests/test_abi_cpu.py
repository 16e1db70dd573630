"""CPU-side checks of the C ABI: the library loads, exports every symbol the
header declares, and its host mesh bookkeeping (RWG edges, basis-function
count, near-pair classification) matches the oracle and the reference."""
import ctypes
import os
import re

import numpy as np
import pytest

from helpers import fixture_surfaces

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _lib():
    from gbem import _lib
    if not os.path.exists(_lib.LIBPATH):
        pytest.skip("libgbem.so not built")
    return _lib


def test_exports_every_declared_symbol():
    L = _lib()
    hdr = open(os.path.join(REPO, "include", "gbem.h")).read()
    declared = sorted(set(re.findall(r"\b(gbem_[a-z_0-9]+)\s*\(", hdr)))
    assert declared, "no declarations found"
    so = ctypes.CDLL(L.LIBPATH)
    missing = [n for n in declared if not hasattr(so, n)]
    assert not missing, missing
    assert sorted(L.EXPORTS) == declared


def test_edges_match_oracle_and_reference(golden):
    from gbem import RWGGeometry
    from oracle import oracle as ora
    d = golden("ref_pec_s2_w1.npz")
    gs, _ = fixture_surfaces(d)
    G = RWGGeometry(gs)
    assert G.TotalBFs == 480
    E, L = G.edges(0)
    Eo, Lo = ora.Surface(d["V0"], d["P0"]).edges()
    assert np.array_equal(E, Eo)
    assert np.allclose(L, Lo, rtol=0, atol=0)


def test_dielectric_bf_count_and_near_pairs(golden):
    from gbem import RWGGeometry
    d = golden("ref_diel_s1_w2.npz")
    gs, _ = fixture_surfaces(d)
    G = RWGGeometry(gs)
    assert G.TotalBFs == 2 * 120
    c = G.near_counts()
    # 80 panels: 80 self pairs, 120 common edges, common vertices: 12*10 + 30*... > 0
    assert c[3] == 80 and c[2] == 120 and c[1] > 0 and c[0] > 0


def test_bad_mesh_is_rejected():
    from gbem import GbemError, RWGGeometry
    V = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 1]], dtype=float)
    # three panels share edge (0,1): non-manifold
    P = np.array([[0, 1, 2], [1, 0, 3], [0, 1, 4]], dtype=np.int32)
    with pytest.raises(GbemError) as e:
        RWGGeometry([{"V": V, "P": P, "material": None}])
    assert "EMESH" in str(e.value)
    with pytest.raises(GbemError):
        RWGGeometry([{"V": V, "P": np.array([[0, 1, 9]], dtype=np.int32), "material": None}])
