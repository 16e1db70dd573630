"""The CPU oracle against the reference: its own unit-test goldens
(unitTests/unit-test-PPIs.cc:70-107) and outputs of the reference built from
its sources (fixtures made by tests/golden/make_golden.py)."""
import numpy as np
import pytest

from oracle import oracle as ora

# per-branch tolerances (relative to the larger of |H0|, |H1| scale), set by the
# reference's own quadrature: LO/HO are fixed rules (bitwise formula), TD uses
# adaptive cubature to 1e-10 (ncv=3) or at most 1000 evaluations (ncv=1,2),
# desingularised pairs use FIPPIs from adaptive cubature at rel 1e-6 / 1e-5.
# the 3-D common-vertex Taylor-Duffy cubature is capped at 1000 evaluations
# (PanelPanelInteractions.cc via InitTaylorDuffyArgs, TaylorDuffy.cc:268-272);
# at |k r| ~ 10 it stops near 3e-4, while this oracle converges to 1e-12
# (checked by raising its order from 14 to 40 points per dimension).
TOL = {("LO", 0): 1e-12, ("HO", 0): 5e-7, ("TD", 3): 1e-9, ("TD", 2): 1e-6, ("TD", 1): 5e-4,
       ("DESING", 0): 1e-6, ("DESING", 1): 1e-6, ("DESING", 2): 1e-7}


def test_unit_ppi_goldens(golden):
    d = golden("ppi_unit.npz")
    S = ora.Surface(d["V"], d["P"])
    for c, exact, ref in zip(d["cases"], d["exact"], d["ref"]):
        pa, qa, pb, qb, kr, ki = c
        H, alg, ncv = S.ppi(int(pa), int(qa), int(pb), int(qb), kr + 1j * ki)
        scale = max(abs(exact[0]), 1e-300)
        # the unit test compares after rounding to float; the goldens carry 10 digits
        assert np.abs(H[0] - exact[0]) <= 2e-6 * scale + 1e-30
        if abs(exact[1]) > 0:
            assert abs(H[1] - exact[1]) <= 2e-6 * abs(exact[1]) + 1e-7 * scale
        # and against the built reference at its own branch tolerance
        tol = TOL[(ora.ALG_NAMES[alg], ncv)]
        assert np.abs(H - ref).max() <= tol * np.abs(ref).max() + 1e-300


def test_ppi_all_branches(golden):
    d = golden("ref_ppi_s2.npz")
    S = ora.Surface(d["V"], d["P"])
    worst = {}
    for c, Href, alg_ref, ncv_ref in zip(d["cases"], d["H"], d["alg"], d["ncv"]):
        pa, qa, pb, qb, kr, ki = c
        H, alg, ncv = S.ppi(int(pa), int(qa), int(pb), int(qb), kr + 1j * ki)
        assert (alg, ncv) == (alg_ref, ncv_ref)
        key = (ora.ALG_NAMES[alg], ncv)
        err = np.abs(H - Href).max() / np.abs(Href).max()
        worst[key] = max(worst.get(key, 0.0), err)
    for key, err in worst.items():
        assert err <= TOL[key], (key, err)
    assert {k[0] for k in worst} == {"LO", "HO", "TD", "DESING"}


def test_fippi_against_reference(golden):
    d = golden("ref_fippi_s2.npz")
    S = ora.Surface(d["V"], d["P"])
    for (pa, pb), ncv_ref, data in zip(d["pairs"], d["ncv"], d["data"]):
        if ncv_ref == 3:
            continue  # common-triangle pairs never use FIPPIs (Taylor-Duffy instead)
        out, ncv, order = S.qifippi(int(pa), int(pb))
        assert ncv == ncv_ref
        scale = np.abs(data).max()
        # reference: hcubature rel 1e-6 (ncv=0), Taylor-Duffy V2P0 rel 1e-5
        assert np.abs(out - data).max() <= (2e-6 if ncv == 0 else 2e-5) * scale


def test_edges_match_reference(golden):
    d = golden("ref_pec_s2_w1.npz")
    S = ora.Surface(d["V0"], d["P0"])
    E, L = S.edges()
    assert E.shape == (480, 8)
    # Euler characteristic of a closed sphere: V - E + F = 2
    assert len(d["V0"]) - len(E) + len(d["P0"]) == 2
    assert np.all(E[:, 0] < E[:, 1]) and np.all(E[:, 5] >= 0)


def _geometry(d):
    n = int(d["objects"])
    surfs, regs, pec, eps, mu = [], [], [], [1.0], [1.0]
    for i in range(n):
        V = d["V%d" % i] + d["disp%d" % i]
        surfs.append(ora.Surface(V, d["P%d" % i]))
        mat = str(d["mat%d" % i])
        if mat == "PEC":
            regs.append((0, -1)); pec.append(True)
        else:
            from gbem.api import Material
            m = Material.parse(mat)
            eps.append(m.eps); mu.append(m.mu)
            regs.append((0, len(eps) - 1)); pec.append(False)
    return surfs, regs, pec, eps, mu


@pytest.mark.parametrize("case", ["diel_s1_w2", "pec2_s1_xi", "pec_s2_w1"])
def test_matrix_against_reference(golden, case):
    d = golden("ref_%s.npz" % case)
    surfs, regs, pec, eps, mu = _geometry(d)
    w = d["omega"][0] + 1j * d["omega"][1]
    M = ora.assemble(surfs, regs, pec, w, eps, mu)
    Mref = d["M"] if "M" in d.files else None
    if Mref is None:
        cols = d["cols"]
        err = np.abs(M[:, cols] - d["Mcols"]).max() / np.abs(d["Mcols"]).max()
    else:
        err = np.abs(M - Mref).max() / np.abs(Mref).max()
    # entries carry the reference's near-field quadrature error (<= ~1e-7 of
    # the largest entry); far-field entries agree to rounding
    assert err < 2e-7, err


def test_matrix_short_wavelength_against_reference(golden):
    """kR = 12, eps = 4+0.1i: touching pairs take Taylor-Duffy with the full
    kernel; the reference caps that cubature at 1000 evaluations
    (TaylorDuffy.cc:263-272), so its entries carry ~1e-6 of the largest."""
    d = golden("ref_diel_s1_w12.npz")
    surfs, regs, pec, eps, mu = _geometry(d)
    w = d["omega"][0] + 1j * d["omega"][1]
    M = ora.assemble(surfs, regs, pec, w, eps, mu)
    err = np.abs(M - d["M"]).max() / np.abs(d["M"]).max()
    assert err < 2e-6, err


@pytest.mark.parametrize("case", ["pec_s2_w1", "diel_s1_w2"])
def test_emt_scattered_power_against_reference(golden, case):
    """EMT scattered power of the reference's own solutions (GetPFT): the
    oracle's restatement from GC[0], GC[1] agrees to the reference's
    near-field quadrature level."""
    d = golden("ref_%s.npz" % case)
    surfs, regs, pec, eps, mu = _geometry(d)
    w = d["omega"][0] + 1j * d["omega"][1]
    j = 0
    while "kn%d" % j in d.files:
        ps = ora.emt_pscat(surfs[0], pec[0], w, d["kn%d" % j])
        assert abs(ps - d["pft%d" % j][1]) < 2e-6 * abs(d["pft%d" % j][1]), (j, ps, d["pft%d" % j])
        j += 1


def test_mie_oracle_against_reference_tables():
    """The Mie oracle (oracle/mie.py) reproduces the reference's sphere power
    tables (unitTests/unit-test-PFT.cc:77-130: R = 1 um, PEC, SiO2 and gold
    at omega = 0.01, 0.1, 1) to their 7 printed digits."""
    import json
    import os
    from oracle import mie
    with open(os.path.join(os.path.dirname(__file__), "golden", "mie_pft_tables.json")) as f:
        tables = json.load(f)["tables"]
    for name, rows in tables.items():
        for w, er, ei, pabs, pscat, _, _ in rows:
            pec = name.startswith("PEC")
            a, s = mie.powers(w, eps=None if pec else complex(er, ei), pec=pec)
            assert abs(s - pscat) < 1e-6 * pscat, (name, w, s, pscat)
            if pec:
                assert abs(a) < 1e-20
            else:
                assert abs(a - pabs) < 1e-6 * pabs, (name, w, a, pabs)


def test_column_assembly_equals_full_assembly():
    """oracle.assemble_cols (whole columns of matrices too large to assemble
    on the CPU) gives the columns of oracle.assemble entry for entry: a
    dielectric sphere, a PEC sphere, and a PEC + dielectric pair (mixed 1x1 /
    2x2 stamping, mirrored blocks)."""
    from gbem import mesh
    V, P = mesh.icosphere(1)
    S = ora.Surface(V, P)
    S2 = ora.Surface(V + [0.0, 0.0, 3.0], P)
    cases = [([S], [(0, 1)], [False], 2.0, [1.0, 2.25 + 0.01j], [1.0, 1.0]),
             ([S], [(0, -1)], [True], 1.0, [1.0], [1.0]),
             ([S, S2], [(0, -1), (0, 1)], [True, False], 1.5, [1.0, 4 + 0.1j], [1.0, 1.0])]
    for args in cases:
        M = ora.assemble(*args)
        cols = [0, 1, 2, 17, 61, M.shape[0] // 2, M.shape[0] - 1]
        assert np.array_equal(ora.assemble_cols(*args, cols), M[:, cols])


def test_stripe_assembly_equals_upper_triangle():
    """oracle.assemble_stripe over a partition of the column edges gives the
    upper triangle of oracle.assemble (the slices the CPU baseline times)."""
    from gbem import mesh
    V, P = mesh.icosphere(1)
    S = ora.Surface(V, P)
    for pec in (False, True):
        eps = [1.0] if pec else [1.0, 2.25 + 0.01j]
        mu = [1.0] * len(eps)
        M = ora.assemble([S], [(0, -1 if pec else 1)], [pec], 2.0, eps, mu)
        ne = S.edges()[0].shape[0]
        Ms = np.zeros_like(M, order="F")
        for a, b in ((0, 7), (7, 40), (40, ne)):
            ora.assemble_stripe(S, pec, 2.0, eps, mu, a, b, Ms)
        assert np.array_equal(np.triu(Ms), np.triu(M))
