"""The FIPPI cache file of the reference (FIPPICache.cc:195-400), host side:
every near pair of the mesh the reference assembled finds its record in the
cache file the reference itself wrote -- the canonical vertex order and the
15-float keys match its own (CanonicallyOrderVertices, AssessPanelPair.cc:
342-455) -- and malformed files are refused."""
import os

import numpy as np
import pytest

from conftest import GOLDEN


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


def test_reference_cache_keys_match(clean_cache):
    from gbem.api import CacheSize, PreloadCache
    path = os.path.join(GOLDEN, "ref_fippi_cache_s1.bin")
    PreloadCache(path)
    assert CacheSize() == (os.path.getsize(path) - 11) // 352
    G = _geometry()
    hits, misses = G.cache_lookup_stats()
    nc = G.near_counts()
    assert hits == nc[0] + nc[1] + nc[2] and misses == 0  # common-triangle pairs use no FIPPIs


def test_store_writes_the_reference_format(clean_cache, tmp_path):
    from gbem.api import CacheSize, ClearCache, PreloadCache, StoreCache
    PreloadCache(os.path.join(GOLDEN, "ref_fippi_cache_s1.bin"))
    n = CacheSize()
    out = tmp_path / "copy.cache"
    StoreCache(str(out))
    raw = out.read_bytes()
    assert raw[:11] == b"FIPPICACHE\x00" and (len(raw) - 11) % 352 == 0 and (len(raw) - 11) // 352 == n
    ClearCache()
    PreloadCache(str(out))
    assert CacheSize() == n
    assert _geometry().cache_lookup_stats()[1] == 0


def test_malformed_files_are_refused(clean_cache, tmp_path):
    from gbem._lib import GbemError
    from gbem.api import CacheSize, PreloadCache
    bad = tmp_path / "bad.cache"
    bad.write_bytes(b"NOTACACHE\x00\x00" + bytes(352))
    with pytest.raises(GbemError):
        PreloadCache(str(bad))
    short = tmp_path / "short.cache"
    short.write_bytes(b"FIPPICACHE\x00" + bytes(351))
    with pytest.raises(GbemError):
        PreloadCache(str(short))
    assert CacheSize() == 0


def test_reference_reads_this_librarys_cache(tmp_path):
    """The reference itself preloads the cache file this library wrote
    (tests/golden/make_gbem_cache.py, on a GPU) and assembles with it: every
    lookup hits, and the matrix equals its cold one to the accuracy gap of the
    two sides' static integrals (the reference's adaptive cubature)."""
    import subprocess
    from conftest import REPO
    refdump = os.path.join(REPO, "oracle", "_ref", "refdump")
    cache = os.path.join(GOLDEN, "gbem_fippi_cache_s1.bin")
    if not (os.path.exists(refdump) and os.path.exists(cache)):
        pytest.skip("needs the reference build (oracle/ref) and the cache fixture")
    from gbem.mesh import write_msh
    m = np.load(os.path.join(GOLDEN, "ref_fippi_cache_s1_mesh.npz"))
    write_msh(str(tmp_path / "sph.msh"), m["V"], m["P"])
    (tmp_path / "s.scuffgeo").write_text("OBJECT sph\n  MESHFILE sph.msh\n  MATERIAL CONST_EPS_2.25+0.01i\nENDOBJECT\n")

    def matrix(args):
        r = subprocess.run([refdump] + args, cwd=tmp_path, capture_output=True, text=True, check=True)
        b = (tmp_path / args[-1]).read_bytes()
        n = int(np.frombuffer(b[:4], np.int32)[0])
        d = np.frombuffer(b[4:], np.float64)
        return (d[0::2] + 1j * d[1::2]).reshape(n, n, order="F"), r.stdout.split()

    M1, hm = matrix(["cachematrix", "s.scuffgeo", "2", "0", cache, "m1.bin"])
    M0, _ = matrix(["matrix", "s.scuffgeo", "2", "0", "m0.bin"])
    assert int(hm[1]) == 0 and int(hm[0]) > 0  # no misses
    assert np.abs(M1 - M0).max() / np.abs(M0).max() < 1e-7
