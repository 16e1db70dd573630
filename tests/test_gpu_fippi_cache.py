"""The FIPPI cache on the GPU: the reference's own cache file warms this
library's near field (the matrix agrees with the cold one to the reference's
cubature accuracy), and a cache written here and read back reproduces the
cold matrix to rounding."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.fixture
def clean_cache():
    from gbem.api import ClearCache
    ClearCache()
    yield
    ClearCache()


def _geometry():
    from gbem import RWGGeometry
    from gbem.api import Material
    m = np.load(os.path.join(GOLDEN, "ref_fippi_cache_s1_mesh.npz"))
    return RWGGeometry([{"V": m["V"], "P": m["P"], "material": Material(2.25 + 0.01j)}])


def test_reference_cache_warms_the_near_field(clean_cache):
    from gbem.api import PreloadCache
    M0 = _geometry().AssembleBEMMatrix(2.0).numpy()
    PreloadCache(os.path.join(GOLDEN, "ref_fippi_cache_s1.bin"))
    G = _geometry()
    assert G.cache_lookup_stats()[1] == 0
    M1 = G.AssembleBEMMatrix(2.0).numpy()
    d = np.abs(M1 - M0).max() / np.abs(M0).max()
    print("reference cache vs cold near table: max entry difference %.2e of max |M|" % d)
    # the reference's static integrals: adaptive cubature to 1e-6 (disjoint
    # pairs) and 1e-5 (touching pairs, Taylor-Duffy V2P0)
    assert 0 < d < 2e-5


def test_stored_cache_round_trip(clean_cache, tmp_path):
    from gbem.api import CacheSize, ClearCache, PreloadCache, StoreCache
    G0 = _geometry()
    M0 = G0.AssembleBEMMatrix(2.0).numpy()
    path = str(tmp_path / "gbem.cache")
    StoreCache(path)
    nc = G0.near_counts()
    # each pair in both panel orders, as the reference looks pairs up
    assert nc[0] + nc[1] + nc[2] < CacheSize() <= 2 * (nc[0] + nc[1] + nc[2])
    del G0
    ClearCache()
    PreloadCache(path)
    G1 = _geometry()
    assert G1.cache_lookup_stats()[1] == 0
    M1 = G1.AssembleBEMMatrix(2.0).numpy()
    d = np.abs(M1 - M0).max() / np.abs(M0).max()
    print("stored and reloaded near table: max entry difference %.2e" % d)
    assert d < 1e-13
