#!/usr/bin/env python3
"""Generate the golden fixtures under tests/golden/ from the reference itself.

Runs only where the reference tree is present (it reads unitTests/ from it and
drives the reference build made by oracle/ref/Makefile, oracle/_ref/refdump).
The fixtures it writes are small and committed; tests never read the reference
tree at run time.

  python tests/golden/make_golden.py --ref <reference source tree>

Fixtures:
  ppi_unit.npz     the 12 known-answer panel-panel cases of the reference's own
                   unit test (unitTests/unit-test-PPIs.cc:70-107 values and the
                   case list at :171-339), on the 4 panels of
                   unitTests/UnitTestSphere_R0P75_414.msh they use, together with
                   the values the built reference returns for them.
  ref_ppi_s2.npz   reference panel-panel integrals on the subdivision-2 icosphere,
                   sampled over every algorithm branch.
  ref_fippi_s2.npz reference Q-independent FIPPI data for near pairs.
  ref_<case>.npz   reference BEM matrices (full or a column sample), plane-wave
                   right-hand sides, solutions and EMT powers for small geometries.
  ref_<case>_grad.npz, ref_<case>_torque.npz  surface blocks with their
                   derivatives for displacements (GradM) and rotations (dMdT).
  ref_fippi_cache_s1.bin  the reference's own FIPPI cache file for the s=1
                   dielectric sphere (with its mesh, ref_fippi_cache_s1_mesh.npz).
  mie_pft_tables.json  the reference's tables of sphere powers (R = 1 um, PEC,
                   SiO2, gold at omega = 0.01, 0.1, 1; unitTests/unit-test-PFT.cc:
                   77-130), read from the test source as text: they pin the Mie
                   oracle (oracle/mie.py).
"""
import argparse
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "scuff-em_gb300"))
sys.path.insert(0, REPO)
from gbem.mesh import icosphere, read_msh, write_msh  # noqa: E402
from oracle import oracle  # noqa: E402

REFDUMP = os.path.join(REPO, "oracle", "_ref", "refdump")
CAS3D = os.path.join(REPO, "oracle", "_ref", "scuff-cas3D")


def run(args, cwd):
    r = subprocess.run([REFDUMP] + [str(a) for a in args], cwd=cwd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("refdump %s failed: %s %s" % (args[0], r.stdout, r.stderr))
    return r.stdout


def read_cbin(path):
    with open(path, "rb") as f:
        n = int(np.frombuffer(f.read(4), dtype=np.int32)[0])
        d = np.frombuffer(f.read(), dtype=np.float64)
    z = d[0::2] + 1j * d[1::2]
    return z.reshape(n, -1, order="F") if z.size == n * n else z


def geo_file(tmp, name, objects):
    """objects: list of (meshname, V, P, material-or-None, displacement)."""
    lines = []
    for (mname, V, P, mat, disp) in objects:
        write_msh(os.path.join(tmp, mname + ".msh"), V, P)
        lines.append("OBJECT %s\n  MESHFILE %s.msh\n" % (mname, mname))
        if mat is not None:
            lines.append("  MATERIAL %s\n" % mat)
        if disp is not None:
            lines.append("  DISPLACED %r %r %r\n" % tuple(disp))
        lines.append("ENDOBJECT\n\n")
    p = os.path.join(tmp, name + ".scuffgeo")
    with open(p, "w") as f:
        f.write("".join(lines))
    return p


def unit_ppi(ref, tmp):
    src = open(os.path.join(ref, "unitTests", "unit-test-PPIs.cc")).read()
    block = src[src.index("cdouble ExactHValues[]"):src.index("cdouble ExactGradHValues[]")]
    vals = re.findall(r"cdouble\(\s*([-+0-9.eE]+)\s*,\s*([-+0-9.eE]+)\s*\)", block)
    exact = np.array([float(a) + 1j * float(b) for a, b in vals]).reshape(12, 2)
    V, P = read_msh(os.path.join(ref, "unitTests", "UnitTestSphere_R0P75_414.msh"))
    keep = [0, 223, 65, 66]
    vids = sorted(set(P[keep].ravel().tolist()))
    vmap = {v: i for i, v in enumerate(vids)}
    Vm = V[vids]
    Pm = np.array([[vmap[v] for v in P[p]] for p in keep], dtype=np.int32)
    pidx = {0: 0, 223: 1, 65: 2, 66: 3}
    pairs = [(0, 0, 223, 0), (0, 0, 65, 0), (0, 0, 66, 0), (0, 0, 0, 0)]
    ks = [0.1, 5.0, 5.0 + 20.0j]
    cases, lines = [], []
    for (a, qa, b, qb) in pairs:
        for k in ks:
            cases.append((pidx[a], qa, pidx[b], qb, k.real, np.imag(k)))
            lines.append("%d %d %d %d %r %r\n" % (a, qa, b, qb, np.real(k), np.imag(k)))
    lst = os.path.join(tmp, "ut.txt")
    open(lst, "w").write("".join(lines))
    import shutil
    shutil.copy(os.path.join(ref, "unitTests", "UnitTestSphere_R0P75_414.msh"), tmp)
    shutil.copy(os.path.join(ref, "unitTests", "PECSphere_R0P75_414.scuffgeo"), tmp)
    run(["ppi", "PECSphere_R0P75_414.scuffgeo", 0, lst, "ut_out.txt"], tmp)
    out = np.loadtxt(os.path.join(tmp, "ut_out.txt"))
    refH = np.stack([out[:, 0] + 1j * out[:, 1], out[:, 2] + 1j * out[:, 3]], axis=1)
    np.savez_compressed(os.path.join(HERE, "ppi_unit.npz"), V=Vm, P=Pm, cases=np.array(cases),
                        exact=exact, ref=refH, alg=out[:, 4].astype(np.int32), ncv=out[:, 5].astype(np.int32))


def ppi_sample(tmp, V, P, name, rng):
    geo = geo_file(tmp, name, [(name, V, P, None, None)])
    c = V[P].mean(axis=1)
    r = np.max(np.linalg.norm(V[P] - c[:, None, :], axis=2), axis=1)
    npan = len(P)
    lines, rows = [], []
    # near pairs of every kind, plus far pairs
    d = np.linalg.norm(c[:, None, :] - c[None, :, :], axis=2) / np.maximum(r[:, None], r[None, :])
    near = np.argwhere(d <= 4.0)
    far = np.argwhere(d > 4.0)
    sel = np.concatenate([near[rng.choice(len(near), 300, replace=False)],
                          far[rng.choice(len(far), 100, replace=False)]])
    ks = [1.0, 2.0 + 0.0066j, 3.0 + 0.01j, 1j * 2.0, 25.0, 40.0 + 1.0j]
    for (a, b) in sel:
        for k in ks:
            qa, qb = rng.integers(0, 3), rng.integers(0, 3)
            lines.append("%d %d %d %d %r %r\n" % (a, qa, b, qb, np.real(k), np.imag(k)))
            rows.append((a, qa, b, qb, np.real(k), np.imag(k)))
    lst = os.path.join(tmp, name + "_ppi.txt")
    open(lst, "w").write("".join(lines))
    run(["ppi", os.path.basename(geo), 0, lst, name + "_ppi_out.txt"], tmp)
    out = np.loadtxt(os.path.join(tmp, name + "_ppi_out.txt"))
    H = np.stack([out[:, 0] + 1j * out[:, 1], out[:, 2] + 1j * out[:, 3]], axis=1)
    np.savez_compressed(os.path.join(HERE, "ref_ppi_%s.npz" % name), V=V, P=P, cases=np.array(rows), H=H,
                        alg=out[:, 4].astype(np.int32), ncv=out[:, 5].astype(np.int32), rrel=out[:, 6])
    # FIPPI data for the near pairs (reference conventions)
    nl = [(a, b) for (a, b) in near[rng.choice(len(near), 200, replace=False)]]
    lst = os.path.join(tmp, name + "_fip.txt")
    open(lst, "w").write("".join("%d %d\n" % ab for ab in nl))
    run(["fippi", os.path.basename(geo), 0, lst, name + "_fip_out.txt"], tmp)
    out = np.loadtxt(os.path.join(tmp, name + "_fip_out.txt"))
    np.savez_compressed(os.path.join(HERE, "ref_fippi_%s.npz" % name), V=V, P=P, pairs=np.array(nl),
                        ncv=out[:, 0].astype(np.int32), data=out[:, 1:34], order=out[:, 34:40].astype(np.int32))


def matrix_case(tmp, name, objects, omega, pw=None, cols=None):
    geo = geo_file(tmp, name, objects)
    run(["matrix", os.path.basename(geo), np.real(omega), np.imag(omega), name + ".bin"], tmp)
    M = read_cbin(os.path.join(tmp, name + ".bin"))
    out = {"omega": np.array([np.real(omega), np.imag(omega)])}
    for i, (mname, V, P, mat, disp) in enumerate(objects):
        out["V%d" % i] = V
        out["P%d" % i] = P
        out["mat%d" % i] = np.array(mat if mat else "PEC")
        out["disp%d" % i] = np.array(disp if disp is not None else [0.0, 0.0, 0.0])
    if cols is None:
        out["M"] = M
    else:
        out["cols"] = np.array(cols)
        out["Mcols"] = M[:, cols]
        out["diag"] = np.diag(M).copy()
    if pw is not None:
        for j, (E0, nh) in enumerate(pw):
            args = [np.real(omega), np.imag(omega)] + list(E0) + list(nh)
            run(["rhs", os.path.basename(geo)] + args + [name + "_rhs%d.bin" % j], tmp)
            s = run(["pft", os.path.basename(geo)] + args + [name + "_kn%d.bin" % j], tmp)
            out["rhs%d" % j] = read_cbin(os.path.join(tmp, name + "_rhs%d.bin" % j))
            out["kn%d" % j] = read_cbin(os.path.join(tmp, name + "_kn%d.bin" % j))
            t = s.split()
            out["pft%d" % j] = np.array([float(t[3]), float(t[5]), float(t[7])])
            out["pw%d" % j] = np.array(list(E0) + list(nh), dtype=np.float64)
    out["objects"] = np.array(len(objects))
    np.savez_compressed(os.path.join(HERE, "ref_%s.npz" % name), **out)


def read_rects(path, count):
    out = []
    with open(path, "rb") as f:
        for _ in range(count):
            nr, nc = np.frombuffer(f.read(8), dtype=np.int32)
            d = np.frombuffer(f.read(16 * nr * nc), dtype=np.float64)
            out.append((d[0::2] + 1j * d[1::2]).reshape(nr, nc, order="F"))
    return out


def grad_case(tmp, name, objects, omega, blocks):
    """Surface blocks and their gradients d/dx_mu (AssembleBEMMatrixBlock with
    GradM, the cas3D path) for each (nsa, nsb) in blocks."""
    geo = geo_file(tmp, name, objects)
    out = {"omega": np.array([np.real(omega), np.imag(omega)])}
    for i, (mname, V, P, mat, disp) in enumerate(objects):
        out["V%d" % i] = V
        out["P%d" % i] = P
        out["mat%d" % i] = np.array(mat if mat is not None else "PEC")
        out["disp%d" % i] = np.array(disp if disp is not None else (0.0, 0.0, 0.0))
    for (a, b) in blocks:
        fn = os.path.join(tmp, "%s_%d%d.bin" % (name, a, b))
        run(["gradblock", os.path.basename(geo), np.real(omega), np.imag(omega), a, b, fn], tmp)
        M, gx, gy, gz = read_rects(fn, 4)
        out["M%d%d" % (a, b)] = M
        out["G%d%d" % (a, b)] = np.stack([gx, gy, gz])
    out["objects"] = np.array(len(objects))
    np.savez_compressed(os.path.join(HERE, "ref_%s.npz" % name), **out)


def torque_case(tmp, name, objects, omega, blocks):
    """Surface blocks and their derivatives dM/dtheta for rotations of the
    row surface about the x, y, z axes through the origin
    (AssembleBEMMatrixBlock with NumTorqueAxes = 3, dMdT, GammaMatrix)."""
    geo = geo_file(tmp, name, objects)
    out = {"omega": np.array([np.real(omega), np.imag(omega)])}
    for i, (mname, V, P, mat, disp) in enumerate(objects):
        out["V%d" % i] = V
        out["P%d" % i] = P
        out["mat%d" % i] = np.array(mat if mat is not None else "PEC")
        out["disp%d" % i] = np.array(disp if disp is not None else (0.0, 0.0, 0.0))
    for (a, b) in blocks:
        fn = os.path.join(tmp, "%s_%d%d.bin" % (name, a, b))
        run(["torqueblock", os.path.basename(geo), np.real(omega), np.imag(omega), a, b, fn], tmp)
        M, tx, ty, tz = read_rects(fn, 4)
        out["M%d%d" % (a, b)] = M
        out["T%d%d" % (a, b)] = np.stack([tx, ty, tz])
    out["objects"] = np.array(len(objects))
    np.savez_compressed(os.path.join(HERE, "ref_%s.npz" % name), **out)


def torque_fixtures(tmp):
    V1, P1 = icosphere(1)
    torque_case(tmp, "pec2_s1_torque", [("a", V1, P1, None, None), ("b", V1, P1, None, (0.0, 0.0, 3.0))], 0.7j,
                [(0, 1), (1, 0)])
    torque_case(tmp, "diel2_s1_torque", [("a", V1, P1, "CONST_EPS_2.25+0.01i", None),
                                         ("b", V1, P1, "CONST_EPS_2.25+0.01i", (0.0, 0.0, 3.0))], 1.5, [(0, 1)])


def gradient_fixtures(tmp):
    V1, P1 = icosphere(1)
    # two PEC spheres, centre gap 3, imaginary frequency: every pair of the
    # inter-sphere block is far (6x6 rule); the self block has near pairs too
    grad_case(tmp, "pec2_s1_grad", [("a", V1, P1, None, None), ("b", V1, P1, None, (0.0, 0.0, 3.0))], 0.7j,
              [(0, 1), (1, 0), (0, 0)])
    # two dielectric spheres (PMCHWT 2x2 stamping), real frequency
    grad_case(tmp, "diel2_s1_grad", [("a", V1, P1, "CONST_EPS_2.25+0.01i", None),
                                     ("b", V1, P1, "CONST_EPS_2.25+0.01i", (0.0, 0.0, 3.0))], 1.5, [(0, 1)])


def mie_tables(ref):
    """Parse the PFTData tables of unitTests/unit-test-PFT.cc (omega, Re eps,
    Im eps, absorbed power, scattered power, z-force, z-torque per row)."""
    import json
    src = open(os.path.join(ref, "unitTests", "unit-test-PFT.cc")).read()
    out = {}
    for name in ("PECPFTData", "SIO2PFTData", "GoldPFTData"):
        body = re.search(name + r"\s*=\s*\{(.*?)\};", src, re.S).group(1)
        nums = [float(x) for x in re.findall(r"[-+]?\d+\.?\d*(?:[eE][-+]?\d+)?", body)]
        out[name] = [nums[i:i + 7] for i in range(0, len(nums), 7)]
    with open(os.path.join(HERE, "mie_pft_tables.json"), "w") as f:
        json.dump({"source": "unitTests/unit-test-PFT.cc:77-130", "columns":
                   ["omega", "eps_re", "eps_im", "p_abs_W", "p_scat_W", "f_z_nN", "tau_z_nN_um"], "tables": out}, f,
                  indent=1)


def cache_fixture(tmp):
    """ref_fippi_cache_s1.bin: the reference's FIPPI cache file (StoreCache)
    after assembling the dielectric s=1 sphere at kR = 2, with the mesh it
    read (ref_fippi_cache_s1_mesh.npz) and its matrix (column sample)."""
    V1, P1 = icosphere(1)
    geo = geo_file(tmp, "cache_s1", [("sph", V1, P1, "CONST_EPS_2.25+0.01i", None)])
    out = os.path.join(HERE, "ref_fippi_cache_s1.bin")
    run(["cache", os.path.basename(geo), 2.0, 0.0, out], tmp)
    V, P = read_msh(os.path.join(tmp, "sph.msh"))
    np.savez_compressed(os.path.join(HERE, "ref_fippi_cache_s1_mesh.npz"), V=V, P=P)


def casimir_fixture(tmp):
    """The reference's own Casimir integrand (scuff-cas3D, unchanged:
    GetCasimirIntegrand, applications/scuff-cas3D/CasimirIntegrand.cc:243-480)
    for two PEC icospheres (subdivision 3, radius 1, centres 3 apart) at the
    20 Gauss-Laguerre nodes x_j scaled by 1/g, for g = 1 (surface gap) and
    g = 3 (centre gap): energy and z-force integrands per xi, read from its
    .byXi file (ref_pec2_s3_casimir.npz)."""
    V3, P3 = icosphere(3)
    write_msh(os.path.join(tmp, "s3.msh"), V3, P3)
    geo = os.path.join(tmp, "pec2_s3.scuffgeo")
    # one mesh file for both bodies, so the reference treats the second as the
    # first's mate and assembles one T block
    with open(geo, "w") as f:
        f.write("OBJECT a\n  MESHFILE s3.msh\nENDOBJECT\n\nOBJECT b\n  MESHFILE s3.msh\n"
                "  DISPLACED 0.0 0.0 3.0\nENDOBJECT\n")
    x, _ = np.polynomial.laguerre.laggauss(20)
    xi = np.concatenate([x / 1.0, x / 3.0])
    with open(os.path.join(tmp, "xi.txt"), "w") as f:
        f.write("".join("%.17g\n" % v for v in xi))
    # the driver reads extra options from stdin when stdin is not a terminal
    # (libhrutil/ProcessOptions.cc:238), so stdin is closed
    r = subprocess.run([CAS3D, "--geometry", os.path.basename(geo), "--XiFile", "xi.txt", "--Energy", "--ZForce"],
                       cwd=tmp, stdin=subprocess.DEVNULL, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("scuff-cas3D failed: %s %s" % (r.stdout, r.stderr))
    rows = [ln.split() for ln in open(os.path.join(tmp, "pec2_s3.byXi")) if ln.strip() and not ln.startswith("#")]
    got = np.array([[float(t) for t in r_[1:4]] for r_ in rows])
    assert np.allclose(got[:, 0], xi, rtol=1e-6), "xi order"
    np.savez_compressed(os.path.join(HERE, "ref_pec2_s3_casimir.npz"), xi=xi, gap=np.repeat([1.0, 3.0], 20),
                        energy=got[:, 1], zforce=got[:, 2], laguerre_x=x)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=oracle.reference_tree(),
                    help="reference source tree (default: SCUFF_REF, or a 'reference' checkout beside the repo)")
    ap.add_argument("--only", choices=["gradients", "torque", "mie", "cache", "casimir"],
                    help="regenerate one group of fixtures only")
    a = ap.parse_args()
    if a.only == "mie":
        mie_tables(a.ref)
        return
    if not os.path.exists(REFDUMP):
        sys.exit("build the reference first: make -C oracle/ref REF=%s" % a.ref)
    if a.only in ("gradients", "torque", "cache", "casimir"):
        with tempfile.TemporaryDirectory() as tmp:
            {"gradients": gradient_fixtures, "torque": torque_fixtures, "cache": cache_fixture,
             "casimir": casimir_fixture}[a.only](tmp)
        return
    rng = np.random.default_rng(0)
    with tempfile.TemporaryDirectory() as tmp:
        unit_ppi(a.ref, tmp)
        V2, P2 = icosphere(2)
        ppi_sample(tmp, V2, P2, "s2", rng)
        V1, P1 = icosphere(1)
        pws = [((1.0, 0.0, 0.0), (0.0, 0.0, 1.0)), ((0.0, 1.0, 0.0), (0.0, 0.0, -1.0))]
        # plain method, small (PEC sphere, s=2, kR = 1): column sample of the 480x480 matrix
        matrix_case(tmp, "pec_s2_w1", [("sph", V2, P2, None, None)], 1.0, pw=pws[:1],
                    cols=list(range(0, 480, 6)))
        # dielectric sphere, s=1, eps = 2.25+0.01i, kR = 2 (PMCHWT, N = 240)
        matrix_case(tmp, "diel_s1_w2", [("sph", V1, P1, "CONST_EPS_2.25+0.01i", None)], 2.0, pw=pws)
        # two PEC spheres (s=1) with centre gap 3, imaginary frequency (real matrix)
        matrix_case(tmp, "pec2_s1_xi", [("a", V1, P1, None, None), ("b", V1, P1, None, (0.0, 0.0, 3.0))], 0.7j)
        # dielectric sphere at a frequency where high-order / Taylor-Duffy branches appear
        matrix_case(tmp, "diel_s1_w12", [("sph", V1, P1, "CONST_EPS_4+0.1i", None)], 12.0)
        gradient_fixtures(tmp)
        torque_fixtures(tmp)
        cache_fixture(tmp)
        casimir_fixture(tmp)
    mie_tables(a.ref)


if __name__ == "__main__":
    main()
