#!/usr/bin/env python3
"""BEM solves/s on one GB300: the mixed-precision solve against the plain FP64
path, on the dielectric-sphere workload (icosphere subdivided 4 times, 5120
panels, 7680 RWG edges, PMCHWT N = 15360, eps = 2.25+0.01i, mu = 1, kR = 2,
4 plane-wave right-hand sides: +-z incidence x/y polarisation).

One step = one full solve: assemble the BEM matrix (warm: the
frequency-independent near-pair table is built once, before timing), factor,
solve the 4 right-hand sides and refine to 1e-10 relative residual.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gbem|reference]

Prints one JSON line.  --impl reference times the CPU implementation of the
path on all host cores (the oracle port of the reference's assembly and
LAPACK's zgetrf/zgetrs; the reference binary built from its sources does not
exist on the GPU host): one full-size solve cut into W + K slices, each step
a real part of it (oracle/cpu_solve.py).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
for p in (REPO, os.path.join(REPO, "scuff-em_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np  # noqa: E402

ZVAC = 376.73031346177
METRIC = "BEM solves/s at N=15360, mixed-prec vs FP64 on one GB300 @<=1e-6 rel err"
PLANE_WAVES = [((1, 0, 0), (0, 0, 1)), ((0, 1, 0), (0, 0, 1)), ((1, 0, 0), (0, 0, -1)), ((0, 1, 0), (0, 0, -1))]

# DRAM read + write bytes per trailing-update launch at N = 15360: one ncu
# capture (dram__bytes_read/write.sum) of the first trailing update of the
# N = 7680 PEC sphere -- 16.4 B per updated complex64 entry -- scaled by the
# entries each of the 59 updates writes (summary under profiles/)
TC_TRAFFIC_BYTES_PER_LAUNCH = 1.28e9
# nominal GB300 CUDA-core rates (the measured-peaks file has HBM and bf16 only)
FP32_PEAK_TFLOPS = 75.0
FP64_PEAK_TFLOPS = 1.25


def far_ppr(G):
    """Far (panel pair, region) units of a one-surface dielectric geometry:
    unordered panel pairs times 2 regions, less the near pairs (rRel <= 4)."""
    npan = G.np_total
    near = sum(G.near_counts())
    return 2 * (npan * (npan + 1) // 2 - near)


def workload(subdiv):
    from gbem import mesh
    V, P = mesh.icosphere(subdiv)
    return V, P


def extinction_power(x, b):
    """P_abs + P_scat = -1/2 ZVAC [Re(K^H b_K) - Re(N^H b_N)] per right-hand side
    (agrees with the reference's EMT powers, GetPFT.cc, on its own solutions)."""
    K, N = x[0::2], x[1::2]
    return -0.5 * ZVAC * (np.real(np.sum(np.conj(K) * b[0::2], axis=0)) - np.real(np.sum(np.conj(N) * b[1::2], axis=0)))


class ClockSampler:
    """nvidia-smi clock and throttle-reason samples during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.rows, self.proc = [], None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                                          "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0],
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([t.strip() for t in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[0]))
                mx = max(mx, float(r[1]))
                for nm, v in zip(names, r[4:8]):
                    if v.strip().lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("bf16_tflops", 1900.0), d.get("hbm_gbs", 6800.0), "measured"
    return 1900.0, 6800.0, "fallback"


def lu_update_flops(N, w=256):
    """Algorithmic flops of the trailing updates of a right-looking LU with
    panel width w: sum over panels of 8 m n w (complex multiply-add)."""
    tot = 0.0
    for c0 in range(0, N, w):
        wc = min(w, N - c0)
        m = N - c0 - wc
        tot += 8.0 * m * m * wc
    return tot


CONFIG_WORKLOAD = "dielectric icosphere s=%d, N=%d, eps=2.25+0.01i, kR=2, %d plane-wave RHS"


def bench_config(subdiv, N, nrhs, world=1, pec=False):
    """The workload dict both arms print (identical keys and values)."""
    wl = CONFIG_WORKLOAD % (subdiv, N, nrhs)
    if pec:
        wl = "PEC icosphere s=%d, N=%d, kR=2, %d plane-wave RHS" % (subdiv, N, nrhs)
    return {"workload": wl,
            "l2": "inputs larger than L2 (C64 matrix %.2f GB, C128 %.2f GB)" % (N * N * 8 / 1e9, N * N * 16 / 1e9),
            "parallelism": "replicas" if world > 1 else "single GPU"}


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count()


def cpu_sample(cores, subdiv=4):
    """A bounded sample of the CPU solve at full size (oracle assembly,
    LAPACK LU; oracle/cpu_solve.py): one column stripe holding 1/64 of the
    upper triangle's edge pairs (assembled cold once to fill the near-pair
    memo, then timed warm) and the LU's first panel steps up to 1/16 of its
    flops, each scaled by its fraction of one solve."""
    from oracle.cpu_solve import SlicedSolve, cpu_model
    job = SlicedSolve(subdiv=subdiv, warm=False)
    eb = job.stripe_bounds(64)
    j = 32  # a stripe in the middle of the column range
    job.assemble(eb[j], eb[j + 1])
    job.M[:] = 0
    ta, fa = job.assemble(eb[j], eb[j + 1])
    kb = job.panel_bounds(16)
    tl, fl = job.factor(kb[0], kb[1])
    t_solve = ta / fa + tl / fl
    return {"value": 1.0 / t_solve, "unit": "solves/s", "cores": cores, "kind": "port", "cpu": cpu_model(),
            "sample": "N=%d at full size: assembly stripe of %.4f of the edge pairs, warm (%.2f s), LU panel steps "
                      "%d-%d = %.4f of the LU flops (%.2f s, blocked zgetrf on a seeded random matrix), scaled "
                      "-> %.1f s per solve" % (job.N, fa, ta, kb[0], kb[1], fl, tl, t_solve)}


def run_reference(args):
    """The reference's CPU path on all host cores (oracle assembly with
    OpenMP, LAPACK LU from OpenBLAS): one full-size solve cut into W + K
    slices.  Every step assembles a column stripe holding 1/(W+K) of the
    upper triangle's edge pairs (warm: the near-pair integrals are memoised
    in the set-up, as the reference's FIPPI cache holds them after the first
    frequency); the K timed steps also run the whole LU, K runs of panel steps
    of about equal flops, and the last one the 4-RHS solve.  Solves/s =
    1 / (assembly time scaled by the timed stripes' pair fraction + LU time +
    solve time).  ms_per_step is the mean wall time of a timed step."""
    if int(os.environ.get("RANK", "0")) != 0:
        return
    # OpenMP threads of the assembly sleep, not spin, while OpenBLAS runs
    os.environ.setdefault("OMP_WAIT_POLICY", "PASSIVE")
    from oracle.cpu_solve import SlicedSolve, cpu_model
    cores = cpu_threads()
    t0 = time.perf_counter()
    job = SlicedSolve(subdiv=args.subdiv)
    t_setup = time.perf_counter() - t0
    W, K = max(0, args.warmup), max(1, args.steps)
    eb = job.stripe_bounds(W + K)
    kb = job.panel_bounds(K)
    t_asm = f_asm = t_lu = f_lu = t_sol = 0.0
    steps_s = []
    for j in range(W + K):
        s0 = time.perf_counter()
        ta, fa = job.assemble(eb[j], eb[j + 1])
        if j >= W:
            i = j - W
            tl, fl = job.factor(kb[i], kb[i + 1])
            t_lu += tl
            f_lu += fl
            if i == K - 1:
                t_sol = job.solve()
            t_asm += ta
            f_asm += fa
            steps_s.append(time.perf_counter() - s0)
    T_asm = t_asm / f_asm
    T = T_asm + t_lu / f_lu + t_sol
    v = 1.0 / T
    ms_step = 1000.0 * statistics.mean(steps_s)
    cb = {"value": v, "unit": "solves/s", "cores": cores, "kind": "port", "cpu": cpu_model(),
          "sample": "one N=%d solve in %d slices: timed steps assembled %.3f of the edge pairs (%.1f s, warm) and "
                    "ran the whole LU (%.1f s, blocked zgetrf on a seeded random matrix, %d panels of 256) and the "
                    "4-RHS zgetrs (%.2f s); solve time %.1f s = assembly %.1f + LU %.1f + solve %.2f; set-up "
                    "(near-pair memo of %d pairs, random matrix) %.1f s untimed"
                    % (job.N, W + K, f_asm, t_asm, t_lu, job.lu.npanels, t_sol, T, T_asm, t_lu / f_lu, t_sol,
                       job.near_pairs, t_setup)}
    print(json.dumps({"metric": METRIC, "value": v, "unit": "solves/s", "n_gpus": args.gpus, "steps": K,
                      "warmup": W, "ms_per_step": ms_step, "higher_is_better": True,
                      "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
                      "impl": "reference", "cpu_baseline": cb,
                      "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                      "config": bench_config(args.subdiv, job.N, 4, args.gpus),
                      "method": "oracle port of the reference's assembly (OpenMP) + LAPACK zgetrf/zgetrs "
                                "(OpenBLAS), FP64",
                      "stages_s_per_solve": {"assembly_warm": T_asm, "lu": t_lu / f_lu, "solve": t_sol}}))


def batch_geometries(seed=0):
    """The batching workload's 48 geometries, seed 0: 24 icospheres of radius
    U[0.5, 1.5] at subdivisions 2, 3, 4 in turn (320-5120 panels) and 24
    rounded cubes of side 1 with U[600, 3000] panels (seeded jittered
    triangulations), each with eps ~ U[1.5, 4] + i U[0, 0.1].  Returns
    [(RWGGeometry, characteristic radius, description)]."""
    from gbem import RWGGeometry, mesh
    from gbem.api import Material
    rng = np.random.default_rng(seed)
    out = []
    for j in range(48):
        eps = complex(rng.uniform(1.5, 4.0), rng.uniform(0.0, 0.1))
        if j % 2 == 0:
            s = 2 + (j // 2) % 3
            R = float(rng.uniform(0.5, 1.5))
            V, P = mesh.icosphere(s, radius=R)
            desc = "icosphere s=%d R=%.3f" % (s, R)
        else:
            npan = int(rng.uniform(600, 3000))
            V, P = mesh.rounded_cube(npan, side=1.0, seed=int(rng.integers(1 << 30)))
            R = 0.5
            desc = "rounded cube %d panels" % len(P)
        out.append((RWGGeometry([{"V": V, "P": P, "material": Material(eps)}]), R, desc))
    return out


def batch_jobs(geoms, nfreq=16):
    """Every geometry swept over nfreq log-spaced kR in [0.1, 5] (omega =
    kR / R), two plane waves (+z incidence, x and y polarisation) per solve."""
    jobs = []
    for G, R, _ in geoms:
        for kR in np.geomspace(0.1, 5.0, nfreq):
            w = kR / R
            B = np.stack([G.AssembleRHSVector(w, e, n) for e, n in PLANE_WAVES[:2]], axis=1)
            jobs.append((G, w, B))
    return jobs


def run_batch(args):
    """Batch throughput on the batching workload (48 geometries x 16
    frequencies = 768 mixed solves, N 960-15360): one step = the whole batch
    through gbem_solve_mixed_batch (up to four concurrent solves); the same
    jobs one at a time are timed once for comparison."""
    from gbem import solve_mixed_batch
    from gbem.api import LUTuning
    geoms = batch_geometries()
    jobs = batch_jobs(geoms)
    t0 = time.perf_counter()
    for _ in range(max(1, args.warmup)):
        solve_mixed_batch(jobs, max_concurrent=4)
    t_warm = time.perf_counter() - t0
    t_bat = []
    for _ in range(max(1, args.steps)):
        t0 = time.perf_counter()
        out = solve_mixed_batch(jobs, max_concurrent=4)
        t_bat.append(time.perf_counter() - t0)
    t0 = time.perf_counter()
    for G, w, B in jobs:
        G.solve_mixed(w, B)
    t_seq = time.perf_counter() - t0
    ns = sorted(G.TotalBFs for G, _, _ in geoms)
    buckets = {}
    for n in ns:
        b = "%d-%d" % ((n // 1024) * 1024, (n // 1024) * 1024 + 1023)
        buckets[b] = buckets.get(b, 0) + 1
    print(json.dumps({"metric": "batched mixed solves/s (48 geometries x 16 frequencies)",
                      "value": len(jobs) / statistics.median(t_bat), "unit": "solves/s", "n_gpus": 1,
                      "steps": len(t_bat), "warmup": max(1, args.warmup), "ms_per_step": 1e3 * statistics.median(t_bat),
                      "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                      "dtype": "c64+fp64-refine", "data": "synthetic",
                      "config": {"workload": "24 icospheres (R 0.5-1.5, s=2,3,4) + 24 rounded cubes (600-3000 panels), "
                                             "eps U[1.5,4]+iU[0,0.1], 16 kR in [0.1,5], 2 RHS, seed 0",
                                 "N_range": [ns[0], ns[-1]], "geometries_per_1024_bucket": buckets,
                                 "jobs": len(jobs), "max_concurrent": 4},
                      "sequential_solves_per_s": len(jobs) / t_seq, "first_pass_s_incl_near_tables": t_warm,
                      "lu_tuning": LUTuning(0),
                      "max_refine_sweeps": max(o[1] for o in out), "max_residual": max(o[2] for o in out)}))


def run_large(args):
    """The large workload: dielectric icosphere s=5 (20480 panels, N = 61440,
    a 30 GB complex64 matrix), eps = 12+0.05i, kR = 4, 8 plane waves
    (+-x, +-y, +-z incidence, two polarisations each, the first 8); mixed
    solve with FP64 refinement.  Prints solves/s and the EMT powers."""
    import torch
    from gbem import RWGGeometry, mesh
    from gbem.api import Material
    V, P = mesh.icosphere(5)
    G = RWGGeometry([{"V": V, "P": P, "material": Material(12 + 0.05j)}])
    w = 4.0
    waves = []
    for d in ((1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)):
        pols = [p for p in ((1, 0, 0), (0, 1, 0), (0, 0, 1)) if np.dot(p, d) == 0]
        waves += [(p, d) for p in pols]
    waves = waves[:8]
    B = np.stack([G.AssembleRHSVector(w, e, n) for e, n in waves], axis=1)
    t0 = time.perf_counter()
    X, it, res = G.solve_mixed(w, B)
    cold = time.perf_counter() - t0
    ts, its = [], []
    for _ in range(max(1, args.steps)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        X, it, res = G.solve_mixed(w, B)
        torch.cuda.synchronize()
        ts.append(time.perf_counter() - t0)
        its.append(it)
    pabs, pscat = G.GetPFT(w, X, RHS=B, precision="mixed")
    t = statistics.median(ts)
    print(json.dumps({"metric": "mixed solves/s at N=61440", "value": 1.0 / t, "unit": "solves/s", "n_gpus": 1,
                      "steps": len(ts), "warmup": 1, "ms_per_step": 1e3 * t, "higher_is_better": True,
                      "scaling": "weak", "vs_baseline": None, "dtype": "c64+fp64-refine", "data": "synthetic",
                      "config": {"workload": "dielectric icosphere s=5, N=%d, eps=12+0.05i, kR=4, 8 plane-wave RHS"
                                             % G.TotalBFs},
                      "cold_first_solve_s": cold, "refine_sweeps": its, "final_rel_residual": res,
                      "absorbed_power": [float(v) for v in pabs], "scattered_power": [float(v) for v in pscat]}))


def run_casimir(args):
    """The Casimir workload: two PEC icospheres (s=3, N = 3840 real), centres
    3 apart; energy and z-force integrands at the 20 Gauss-Laguerre
    frequencies xi = x_j / g (g = 1, the surface gap), and the integrated
    energy and force (sum of weights x integrand).  One step = the 20-point
    sweep."""
    from gbem import mesh
    from gbem.casimir import CasimirIntegrand, laguerre_xi
    V, P = mesh.icosphere(3)
    cas = CasimirIntegrand([{"V": V, "P": P, "material": None}, {"V": V + [0.0, 0.0, 3.0], "P": P, "material": None}])
    xi, wt = laguerre_xi(20, 1.0)
    for _ in range(max(1, args.warmup)):
        cas(float(xi[0]))
    ts = []
    for _ in range(max(1, args.steps)):
        t0 = time.perf_counter()
        vals = [cas(float(x)) for x in xi]
        ts.append(time.perf_counter() - t0)
    E = np.array([v[0] for v in vals])
    F = np.array([v[1] for v in vals])
    t = statistics.median(ts)
    print(json.dumps({"metric": "Casimir integrand points/s (two PEC spheres, N=3840)", "value": len(xi) / t,
                      "unit": "xi/s", "n_gpus": 1, "steps": len(ts), "warmup": max(1, args.warmup),
                      "ms_per_step": 1e3 * t, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                      "dtype": "f64", "data": "synthetic",
                      "config": {"workload": "2 PEC icospheres s=3, centre gap 3, 20 Gauss-Laguerre xi, surface gap 1"},
                      "xi": [float(x) for x in xi], "energy_integrand": E.tolist(), "zforce_integrand": F.tolist(),
                      "energy": float(np.dot(wt, E)), "zforce": float(np.dot(wt, F))}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gbem", choices=["gbem", "reference"])
    ap.add_argument("--subdiv", type=int, default=4)
    ap.add_argument("--pec", action="store_true",
                    help="a PEC sphere instead of the dielectric one (N = 30 * 4^s; for profiling runs)")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--fp64-reps", type=int, default=5, help="plain FP64 solves timed (median reported)")
    ap.add_argument("--workload", default="solve", choices=["solve", "batch", "large", "casimir"],
                    help="solve: the headline N=15360 mixed solve; batch: 48 geometries x 16 frequencies; "
                         "large: the N=61440 sphere; casimir: the two-sphere Casimir sweep")
    args = ap.parse_args()
    if args.pec:
        args.no_fp64 = True  # the accuracy report assumes the dielectric's K/N interleaving
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batch":
        return run_batch(args)
    if args.workload == "large":
        return run_large(args)
    if args.workload == "casimir":
        return run_casimir(args)

    import ctypes
    import torch
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from gbem import RWGGeometry, _lib
    from gbem.api import Material
    from gbem._lib import check, lib

    V, P = workload(args.subdiv)
    G = RWGGeometry([{"V": V, "P": P, "material": None if args.pec else Material(2.25 + 0.01j)}], device=local)
    N = G.TotalBFs
    w = 2.0
    stream = torch.cuda.current_stream()
    check(lib().gbem_geometry_set_stream(G._h, ctypes.c_void_p(stream.cuda_stream)))
    B = np.stack([G.AssembleRHSVector(w, e, n) for e, n in PLANE_WAVES], axis=1)
    nrhs = B.shape[1]
    eps, mu = G.eps_mu(w)
    dB = torch.from_numpy(np.asfortranarray(B).T.copy()).to("cuda")  # nrhs x N row-major == N x nrhs col-major
    dX = torch.zeros_like(dB)
    it, res = ctypes.c_int(), ctypes.c_double()

    def solve_device():
        st = lib().gbem_solve_mixed_device(G._h, w, 0.0, eps.ctypes.data, mu.ctypes.data, nrhs, dB.data_ptr(), N,
                                           dX.data_ptr(), N, 1e-10, 20, ctypes.byref(it), ctypes.byref(res))
        if st not in (_lib.GBEM_OK, _lib.GBEM_ENOCONV):
            check(st)

    hB = torch.from_numpy(np.asfortranarray(B).T.copy()).pin_memory()
    hX = torch.zeros_like(hB).pin_memory()

    def solve_host():
        st = lib().gbem_solve_mixed(G._h, w, 0.0, eps.ctypes.data, mu.ctypes.data, nrhs, hB.data_ptr(), N,
                                    hX.data_ptr(), N, 1e-10, 20, ctypes.byref(it), ctypes.byref(res))
        if st not in (_lib.GBEM_OK, _lib.GBEM_ENOCONV):
            check(st)

    # warm-up: the first call builds the frequency-independent near-pair table
    t0 = time.perf_counter()
    solve_device()
    cold_s = time.perf_counter() - t0
    for _ in range(max(0, args.warmup - 1)):
        solve_device()
    torch.cuda.synchronize()
    lib().gbem_stats(1, None, None)  # reset, enable event timing
    clocks = ClockSampler()
    clocks.start()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    iters = []
    for _ in range(args.steps):
        solve_device()
        iters.append(it.value)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    ck = clocks.stop()
    stage_ms = (ctypes.c_double * 8)()
    stage_n = (ctypes.c_longlong * 8)()
    lib().gbem_stats(0, stage_ms, stage_n)
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    ms_step = ms / args.steps
    value = world * 1000.0 / ms_step
    Xmixed = dX.cpu().numpy().T.copy()
    final_res = res.value

    # end to end through the host-buffer C ABI call
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        solve_host()
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1) / args.steps

    out = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "c64+fp64-refine", "data": "synthetic",
           "config": bench_config(args.subdiv, N, nrhs, world, args.pec),
           "method": "mixed: float-float far field + FP64 near field -> C64, split-BF16 tensor-core LU, "
                     "FP64 refinement to 1e-10",
           "e2e": {"value": world * 1000.0 / e2e_ms, "unit": "solves/s",
                   "h2d_bytes_per_step": int(N * nrhs * 16), "d2h_bytes_per_step": int(N * nrhs * 16)},
           "refine_sweeps": iters, "final_rel_residual": final_res, "cold_first_solve_s": cold_s,
           "clocks": ck}
    names = ["far_field_tiles", "near_singular_pairs", "lu_panels", "lu_trailing_update", "triangular_solves",
             "fp64_residual", "other", "reserved"]
    out["stages_ms_per_step"] = {names[i]: stage_ms[i] / args.steps for i in range(7)}
    out["gpu_launches"] = int(sum(stage_n[i] for i in range(8)))

    # roofline of the dominant stage (tensor-core trailing update of the LU)
    bf16_peak, hbm_peak, peak_kind = measured_peaks()
    upd_flops = lu_update_flops(N)
    gemm_ms = stage_ms[3] / args.steps
    if gemm_ms > 0:
        n_upd = max(1, (N + 255) // 256 - 1)
        ach = upd_flops / (gemm_ms * 1e-3) / 1e12
        # DRAM bytes per trailing-update launch from one ncu capture of this
        # workload; valid for N = 15360 only
        traffic = TC_TRAFFIC_BYTES_PER_LAUNCH if N == 15360 else None
        out["roofline"] = {"bound": "tensor", "achieved": ach, "peak": bf16_peak, "unit": "TFLOP/s",
                           "frac": ach / bf16_peak, "traffic": traffic, "kernel": "tc_gemm_kernel (+split packing)",
                           "launches_per_step": n_upd, "peak_kind": peak_kind,
                           "note": "algorithmic complex flops 8mnk; the split-BF16 form issues 3x that on the "
                                   "tensor pipe"}
    # the assembly's far field (ppair + stamp kernels): far (panel pair,
    # region) units per second, their algorithmic FP32 flops (3600 per unit:
    # 36 kernel samples x 100) against the FP32 pipe, and the HBM traffic
    # the stage must make (the C64 matrix written once, panel tables read)
    far_ms = stage_ms[0] / args.steps
    if far_ms > 0:
        ppr = far_ppr(G)
        fl = ppr * 3600.0
        out["roofline_assembly"] = {
            "kernel": "ppair_kernel + stamp_kernel (far field, float-float)", "bound": "fp32",
            "panel_pairs_per_s": ppr / (far_ms * 1e-3), "far_ppr": ppr,
            "achieved_tflops": fl / (far_ms * 1e-3) / 1e12, "peak_tflops": FP32_PEAK_TFLOPS,
            "frac": fl / (far_ms * 1e-3) / 1e12 / FP32_PEAK_TFLOPS,
            "peak_kind": "nominal FP32 (no measured FP32 figure in MEASURED_PEAKS.json)",
            "hbm_gbs": (N * N * 8 + G.np_total * 64 * 8) / (far_ms * 1e-3) / 1e9, "hbm_peak_gbs": hbm_peak,
            "note": "float-float arithmetic issues ~640 FP32 instructions per sample against the 100-flop "
                    "convention"}
    # solve and refinement: every sweep reads the complex64 factor once (its
    # forward and backward triangular solves) and the complex64 matrix once
    # (the FP64-accurate residual), against the HBM copy bandwidth
    sol_ms = (stage_ms[4] + stage_ms[5]) / args.steps
    if sol_ms > 0 and iters:
        sweeps = statistics.median(iters)
        nbytes = 2 * sweeps * N * N * 8
        out["roofline_solve"] = {
            "kernel": "trsv_coop (4 RHS) + residual_partial_df", "bound": "hbm",
            "bytes_per_step": nbytes, "achieved_gbs": nbytes / (sol_ms * 1e-3) / 1e9, "peak_gbs": hbm_peak,
            "frac": nbytes / (sol_ms * 1e-3) / 1e9 / hbm_peak, "sweeps": sweeps,
            "note": "latency-bound: one grid barrier per 64-row block in each triangular solve"}

    # plain FP64 path (same geometry): assemble C128, LU, solve -- repeated,
    # with its own stage split
    if not args.no_fp64:
        fp64_ms, X64 = [], None
        reps = max(1, args.fp64_reps)
        lib().gbem_stats(1, None, None)
        for r in range(reps):
            M = G.AllocateBEMMatrix()
            torch.cuda.synchronize()
            e0.record(stream)
            G.AssembleBEMMatrix(w, M)
            M.LUFactorize()
            X64 = M.LUSolve(B)
            e1.record(stream)
            torch.cuda.synchronize()
            fp64_ms.append(e0.elapsed_time(e1))
            del M
        lib().gbem_stats(0, stage_ms, stage_n)
        f64_stage = {names[i]: stage_ms[i] / reps for i in range(7)}
        t64 = statistics.median(fp64_ms)
        lu64_ms = f64_stage["lu_panels"] + f64_stage["lu_trailing_update"]
        rel_x = float(np.max(np.linalg.norm(Xmixed - X64, axis=0) / np.linalg.norm(X64, axis=0)))
        p64 = extinction_power(X64, B)
        pmx = extinction_power(Xmixed, B)
        out["fp64"] = {"value": 1000.0 / t64, "unit": "solves/s", "ms_per_solve": t64, "ms_all": fp64_ms,
                       "runs": reps, "stages_ms_per_solve": f64_stage}
        if lu64_ms > 0:
            a64 = 8.0 * N ** 3 / 3.0 / (lu64_ms * 1e-3) / 1e12
            out["fp64"]["roofline_lu"] = {"bound": "fp64", "achieved_tflops": a64, "peak_tflops": FP64_PEAK_TFLOPS,
                                          "frac": a64 / FP64_PEAK_TFLOPS,
                                          "peak_kind": "nominal FP64 (no measured FP64 figure in "
                                                       "MEASURED_PEAKS.json)",
                                          "kernel": "panel_kernel<double> + gemm_simt<double> (8N^3/3 flops)"}
        out["speedup_vs_fp64"] = out["value"] / out["fp64"]["value"]
        out["accuracy"] = {"rel_err_x_vs_fp64": rel_x,
                           "rel_err_extinction_power_vs_fp64": float(np.max(np.abs(pmx - p64) / np.abs(p64))),
                           "extinction_power_fp64": [float(v) for v in p64]}
        # EMT scattered and absorbed power (GetPFT's default method) of both
        # solutions, each with the FP64 exterior-region matrix
        pa64, ps64 = G.GetPFT(w, X64, RHS=B)
        pamx, psmx = G.GetPFT(w, Xmixed, RHS=B)
        out["accuracy"]["rel_err_scattered_power_vs_fp64"] = float(np.max(np.abs(psmx - ps64) / np.abs(ps64)))
        out["accuracy"]["rel_err_absorbed_power_vs_fp64"] = float(np.max(np.abs(pamx - pa64) / np.abs(pa64)))
        out["accuracy"]["scattered_power_fp64"] = [float(v) for v in ps64]
        out["accuracy"]["absorbed_power_fp64"] = [float(v) for v in pa64]
    if not args.no_cpu and rank == 0 and world == 1:
        try:
            out["cpu_baseline"] = cpu_sample(cpu_threads(), args.subdiv)
        except Exception as e:  # the CPU leg is a report, not the measurement
            out["cpu_baseline"] = {"error": str(e)}
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
