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
path (the oracle port of the reference's algorithm; the reference binary
built from its sources does not exist on the GPU host) on all host cores.
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

# DRAM read + write bytes per trailing-update launch at N = 15360, measured by
# ncu (dram__bytes_read.sum + dram__bytes_write.sum, 1 pass) over 48 of the 59
# launches of a factorisation, the 11 smallest estimated from the last captured
# one's bytes per entry (the capture's summary is kept under profiles/)
TC_TRAFFIC_BYTES_PER_LAUNCH = 1.45e9


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


def cpu_sample(cores):
    """Oracle port on the host cores, bounded sample: assembly of the
    subdivision-2 dielectric sphere (N = 960) scaled by the edge-pair count
    ratio (7680/480)^2, plus LAPACK zgetrf at N = 3840 scaled by (15360/3840)^3."""
    from oracle import oracle
    import scipy.linalg as sl
    V, P = workload(2)
    S = oracle.Surface(V, P)
    eps = [1.0, 2.25 + 0.01j]
    t0 = time.perf_counter()
    oracle.assemble([S], [(0, 1)], [False], 2.0, eps, [1.0, 1.0])
    t_asm = time.perf_counter() - t0
    rng = np.random.default_rng(0)
    n_lu = 3840
    A = rng.standard_normal((n_lu, n_lu)) + 1j * rng.standard_normal((n_lu, n_lu))
    t0 = time.perf_counter()
    sl.lu_factor(A, overwrite_a=True, check_finite=False)
    t_lu = time.perf_counter() - t0
    t_solve = (7680.0 / 480.0) ** 2 * t_asm + (15360.0 / n_lu) ** 3 * t_lu
    return {"value": 1.0 / t_solve, "unit": "solves/s", "cores": cores, "kind": "port",
            "sample": "oracle assembly of the N=960 sphere (%.2f s) x256 + zgetrf N=3840 (%.2f s) x64 "
                      "-> %.1f s per N=15360 solve" % (t_asm, t_lu, t_solve)}


def run_reference(args):
    cores = os.cpu_count()
    if int(os.environ.get("RANK", "0")) != 0:
        return
    vals = []
    for _ in range(max(1, args.steps)):
        vals.append(cpu_sample(cores))
    v = statistics.median([c["value"] for c in vals])
    cb = dict(vals[-1])
    cb["value"] = v
    print(json.dumps({"metric": METRIC, "value": v, "unit": "solves/s", "n_gpus": args.gpus, "steps": args.steps,
                      "warmup": args.warmup, "ms_per_step": 1000.0 / v, "higher_is_better": True,
                      "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
                      "impl": "reference", "cpu_baseline": cb,
                      "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                      "config": {"workload": "dielectric icosphere s=4, N=15360, eps=2.25+0.01i, kR=2, 4 RHS",
                                 "impl_note": "oracle port of the reference algorithm, OpenMP + LAPACK"}}))


def batch_jobs(seed=0):
    """A synthetic batch in the shape of the batching workload: icospheres of
    radius 0.5-1.5 at subdivisions 2-3, eps ~ U[1.5, 4] + i U[0, 0.1], each
    swept over log-spaced kR in [0.1, 5], two plane waves per solve."""
    from gbem import RWGGeometry, mesh
    from gbem.api import Material
    rng = np.random.default_rng(seed)
    jobs = []
    for g in range(8):
        s = 2 + g % 2
        R = rng.uniform(0.5, 1.5)
        V, P = mesh.icosphere(s, radius=R)
        eps = complex(rng.uniform(1.5, 4.0), rng.uniform(0.0, 0.1))
        G = RWGGeometry([{"V": V, "P": P, "material": Material(eps)}])
        for kR in np.geomspace(0.1, 5.0, 4):
            w = kR / R
            B = np.stack([G.AssembleRHSVector(w, e, n) for e, n in PLANE_WAVES[:2]], axis=1)
            jobs.append((G, w, B))
    return jobs


def run_batch(args):
    """Batch throughput: the same jobs one at a time and as one batch of up to
    four concurrent solves (gbem_solve_mixed_batch).  A 'step' is the whole
    batch; value = solves/s of the batched form."""
    import time
    from gbem import solve_mixed_batch
    jobs = batch_jobs()
    for _ in range(max(args.warmup, 3) // 3):
        solve_mixed_batch(jobs, max_concurrent=4)
    t_seq, t_bat = [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        for G, w, B in jobs:
            G.solve_mixed(w, B)
        t_seq.append(time.perf_counter() - t0)
        t0 = time.perf_counter()
        out = solve_mixed_batch(jobs, max_concurrent=4)
        t_bat.append(time.perf_counter() - t0)
    ns = [G.TotalBFs for G, _, _ in jobs]
    print(json.dumps({"metric": "batched mixed solves/s (frequency sweeps of 8 geometries)", "value": len(jobs) / min(t_bat),
                      "unit": "solves/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
                      "ms_per_step": 1e3 * min(t_bat), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                      "dtype": "c64+fp64-refine", "data": "synthetic",
                      "config": {"workload": "8 dielectric icospheres (s=2,3; R 0.5-1.5) x 4 kR in [0.1, 5], 2 RHS",
                                 "N_range": [min(ns), max(ns)], "jobs": len(jobs), "max_concurrent": 4},
                      "sequential_solves_per_s": len(jobs) / min(t_seq),
                      "max_refine_sweeps": max(o[1] for o in out), "max_residual": max(o[2] for o in out)}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gbem", choices=["gbem", "reference"])
    ap.add_argument("--subdiv", type=int, default=4)
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--workload", default="solve", choices=["solve", "batch"],
                    help="solve: the headline N=15360 mixed solve; batch: a frequency-sweep / multi-geometry batch")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batch":
        return run_batch(args)

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
    G = RWGGeometry([{"V": V, "P": P, "material": Material(2.25 + 0.01j)}], device=local)
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
           "config": {"workload": "dielectric icosphere s=%d, N=%d, eps=2.25+0.01i, kR=2, %d plane-wave RHS"
                                  % (args.subdiv, N, nrhs),
                      "solve": "mixed: FP32 far field + FP64 near field -> C64, split-BF16 tensor-core LU, "
                               "FP64 refinement to 1e-10",
                      "l2": "inputs larger than L2 (C64 matrix %.2f GB)" % (N * N * 8 / 1e9),
                      "parallelism": "replicas" if world > 1 else "single GPU"},
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

    # plain FP64 path (same geometry): assemble C128, LU, solve
    if not args.no_fp64:
        M = G.AllocateBEMMatrix()
        torch.cuda.synchronize()
        e0.record(stream)
        G.AssembleBEMMatrix(w, M)
        M.LUFactorize()
        X64 = M.LUSolve(B)
        e1.record(stream)
        torch.cuda.synchronize()
        fp64_ms = e0.elapsed_time(e1)
        del M
        rel_x = float(np.max(np.linalg.norm(Xmixed - X64, axis=0) / np.linalg.norm(X64, axis=0)))
        p64 = extinction_power(X64, B)
        pmx = extinction_power(Xmixed, B)
        out["fp64"] = {"value": 1000.0 / fp64_ms, "unit": "solves/s", "ms_per_solve": fp64_ms}
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
            out["cpu_baseline"] = cpu_sample(os.cpu_count())
        except Exception as e:  # the CPU leg is a report, not the measurement
            out["cpu_baseline"] = {"error": str(e)}
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
