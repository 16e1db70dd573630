"""The drop-in boundary as the reference's own programs see it: the shim
(scuff-em_gb300/shim/scuff_gbem_shim.cc) compiled against the reference's
headers, and the reference's scuff-scatter and scuff-cas3D relinked,
unchanged, with it ahead of the reference's libraries.  The dynamic linker
must bind the hot-path entry points (AssembleBEMMatrix, AssembleBEMMatrixBlock,
LUFactorize, LUSolve) to the shim, and a run must reach this library.  Needs a
reference source tree (skipped elsewhere); without a GPU the run stops with
the library's error, through the reference's ErrExit."""
import os
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM = os.path.join(REPO, "scuff-em_gb300", "shim")


@pytest.fixture(scope="module")
def built(tmp_path_factory):
    from oracle import oracle
    ref = oracle.reference_tree()
    if not ref:
        pytest.skip("no reference source tree on this machine")
    from gbem import _lib
    if not os.path.exists(_lib.LIBPATH):
        pytest.skip("libgbem.so not built")
    oracle.build_reference(ref)
    r = subprocess.run(["make", "-C", SHIM, "REF=" + ref, "-j4"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    d = tmp_path_factory.mktemp("shim")
    from gbem.mesh import icosphere, write_msh
    V, P = icosphere(1)
    write_msh(str(d / "s1.msh"), V, P)
    (d / "two.scuffgeo").write_text("OBJECT a\n  MESHFILE s1.msh\nENDOBJECT\n\nOBJECT b\n  MESHFILE s1.msh\n"
                                    "  DISPLACED 0.0 0.0 3.0\nENDOBJECT\n")
    (d / "one.scuffgeo").write_text("OBJECT s\n  MESHFILE s1.msh\n  MATERIAL CONST_EPS_2.25\nENDOBJECT\n")
    return d


def _run(exe, args, cwd):
    # every symbol bound at start-up, so the trace lists them whether or not
    # the run gets to call them; the driver reads options from a non-terminal
    # stdin (libhrutil/ProcessOptions.cc:238), so stdin is closed
    tag = "bind_" + exe
    env = dict(os.environ, LD_DEBUG="bindings", LD_BIND_NOW="1", LD_DEBUG_OUTPUT=str(cwd / tag))
    r = subprocess.run([os.path.join(SHIM, "_build", exe)] + args, cwd=cwd, env=env, stdin=subprocess.DEVNULL,
                       capture_output=True, text=True, timeout=600)
    binds = "".join(open(os.path.join(cwd, f)).read() for f in os.listdir(cwd) if f.startswith(tag))
    return r, binds


def _bound_to_shim(binds, sym):
    lines = [ln for ln in binds.splitlines() if sym in ln and "normal symbol" in ln]
    return lines and all("libscuff_gbem_shim.so" in ln.split(" to ")[1] for ln in lines)


def test_cas3d_binds_its_hot_path_to_the_shim(built):
    r, binds = _run("scuff-cas3D-gbem", ["--geometry", "two.scuffgeo", "--Energy", "--ZForce", "--Xi", "0.5"], built)
    assert _bound_to_shim(binds, "RWGGeometry22AssembleBEMMatrixBlock"), binds[-2000:]
    assert _bound_to_shim(binds, "HMatrix11LUFactorize")
    out = r.stdout + r.stderr
    if r.returncode != 0:  # no GPU here: the library's own error, through ErrExit
        assert "AssembleBEMMatrixBlock" in out, out


def test_scatter_binds_its_hot_path_to_the_shim(built):
    r, binds = _run("scuff-scatter-gbem", ["--geometry", "one.scuffgeo", "--Omega", "1.0", "--PWPolarization", "1",
                                           "0", "0", "--PWDirection", "0", "0", "1", "--PFTFile", "out.pft"], built)
    assert _bound_to_shim(binds, "RWGGeometry17AssembleBEMMatrixE"), binds[-2000:]
    assert _bound_to_shim(binds, "HMatrix11LUFactorize") and _bound_to_shim(binds, "HMatrix7LUSolve")
    out = r.stdout + r.stderr
    if r.returncode != 0:
        assert "AssembleBEMMatrix" in out, out
