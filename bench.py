#!/usr/bin/env python
"""bench.py -- IFGF forward-map throughput of the GB300 build on the kite at k = 500.

Workload (the configuration the headline metric is quoted on): Colton-Kress kite
x(t) = (cos t + 0.65 cos 2t - 0.65, 1.5 sin t), k = 500, 512 equal-parameter patches x 16
Fejer nodes (N = 8192), combined-field operator (1/2 I + K - i k S), IFGF with 5 x 5 Chebyshev nodes per cone,
the deepest tree that keeps singular points in the leaf neighbourhood, FP64 (plain form).
A step is one forward map y = A x (singular correction + IFGF far field) on a seeded
mt19937(0) density.  Synthetic geometry, no dataset.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  value: matvecs/s with vectors resident in HBM; e2e: the same
through the C ABI (ifgf2d_apply) with pinned host buffers, copies inside the timed region;
roofline: the dominant phase from live CUDA-event timings; cpu_baseline: the CPU oracle
(single-threaded restatement of the reference path) on a bounded sample.  Multi-GPU runs
are independent replicas (the path has no exchange step); value sums all ranks.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

K_WAVE = 500.0
NPATCH, NP, DELTA = 512, 16, 0.01
METRIC = "IFGF matvecs/s (kite k=500, N=8192, FP64 combined field)"
UNIT = "matvec/s"
WORKLOAD = ("kite k=500, 512 equal patches x 16 Fejer nodes (N=8192), combined field (1/2 I + K - i k S), "
            "IFGF 5x5 cones, FP64")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-solve", action="store_true", help="skip the GMRES solve (for profiler runs)")
    ap.add_argument("--no-batch", action="store_true", help="skip the 64-angle batch (kite k=2000, N=32768)")
    ap.add_argument("--no-obstacles", action="store_true", help="skip the 256-obstacle workload")
    ap.add_argument("--no-large", action="store_true", help="skip the kite k=8000, N=131072 solve")
    ap.add_argument("--no-learned", action="store_true", help="skip the preconditioner comparison (spectral, learned)")
    ap.add_argument("--precond-k", default="2000,8000", help="wavenumbers of the preconditioner comparison (kite, 1.024 k patches)")
    ap.add_argument("--batch-k", type=float, default=2000.0, help="wavenumber of the batch workload (profiling)")
    ap.add_argument("--batch-patches", type=int, default=2048, help="patches of the batch workload (profiling)")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


# ---------------------------------------------------------------- clocks
class ClockSampler:
    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            import tempfile
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "100", "-i", str(self.gpu)], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1])); smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------- workload
def make_ours():
    import ifgf2d_gb300 as G
    fm = G.ForwardMap(DELTA, [G.Kite()], (), 1.0, K_WAVE, Np=NP, patches_per_curve=NPATCH, formulation="combined")
    fm.precomps_and_setup(K_WAVE, 0)
    fm.tuning = fm.autotune()   # per-level launch shapes timed on this problem (cached on disk)
    return G, fm


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def phase_model(wc, N, P, ncones_leaf, nparent):
    """Algorithmic bytes and flops of each apply phase (FP64: complex = 16 B)."""
    C = 16
    near, leaf, prop, interp, cones, sing = (wc["near_pairs"], wc["leaf_evals"], wc["prop_evals"],
                                            wc["interp_evals"], wc["cones"], wc["sing_entries"])
    return {
        "sing_correction": (sing * C + 2 * N * C, sing * 8),
        "intensities": (N * (C + 8 + 8 + C), N * 2),
        "leaf_cones": (leaf * C + N * C + ncones_leaf * P * C, leaf * 8),
        "propagation": (prop * 40 + cones * P * C, prop * (4 * P + 18) + nparent * P * P * 4),
        "near_interp": (near * C + interp * 40 + cones * P * C + 3 * N * C, near * 8 + interp * (4 * P + 18)),
    }


def max_over_ranks(v, world, device):
    """The slowest rank's value (a barrier follows): the whole job is as fast as its slowest replica."""
    if world <= 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.barrier()
    return float(t.item())


def replica_value(world, steps, ms):
    """Whole-job matvecs/s: every replica did `steps` applies in at most `ms` milliseconds."""
    return world * steps / (ms * 1e-3)


# the device results the CPU-baseline leg compares with the oracle (filled by run_ours)
CHECK = {}


def run_ours(args, rank, local_rank, world):
    import torch
    torch.cuda.set_device(local_rank)
    G, fm = make_ours()
    seeded_density = G.seeded_density
    N = fm.total_num_unknowns_
    wc = fm.work_counts()
    L = G._lib.load()
    ext = torch.cuda.ExternalStream(fm.stream())
    x_h = seeded_density(N)
    x = torch.from_numpy(x_h).to("cuda")
    y = torch.empty_like(x)
    torch.cuda.synchronize()
    # warm-up
    for _ in range(max(args.warmup, 3)):
        fm.apply_device(x, y)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank) as clk:
        torch.cuda.synchronize()
        e0.record(ext)
        for _ in range(args.steps):
            fm.apply_device(x, y)
        e1.record(ext)
        torch.cuda.synchronize()
    ms = max_over_ranks(e0.elapsed_time(e1), world, "cuda")
    value = replica_value(world, args.steps, ms)
    # the chosen form: IFGF far field in complex64 (FP32 arithmetic), FP64 singular correction
    for _ in range(max(args.warmup, 3)):
        fm.apply_device(x, y, mixed=True)
    torch.cuda.synchronize()
    e4, e5 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e4.record(ext)
    for _ in range(args.steps):
        fm.apply_device(x, y, mixed=True)
    e5.record(ext)
    torch.cuda.synchronize()
    ms_mixed = e4.elapsed_time(e5)
    y_mixed = y.cpu().numpy()
    fm.apply_device(x, y)
    torch.cuda.synchronize()
    mixed_err = float(np.linalg.norm(y_mixed - y.cpu().numpy()) / np.linalg.norm(y.cpu().numpy()))
    # both forms against the FP64 O(N^2) direct sum with the same singular corrections (the
    # device's own direct map here; the oracle's is compared in the CPU-baseline leg)
    CHECK["density"] = x_h
    CHECK["y_fp64"] = y.cpu().numpy()
    CHECK["y_mixed"] = y_mixed
    y_direct = fm.compute_Ax_unacc(x_h)
    accuracy = {"ifgf_fp64_rel_err_vs_direct": float(np.linalg.norm(y.cpu().numpy() - y_direct) / np.linalg.norm(y_direct)),
                "ifgf_mixed_rel_err_vs_direct": float(np.linalg.norm(y_mixed - y_direct) / np.linalg.norm(y_direct)),
                "mixed_rel_err_vs_fp64_ifgf": mixed_err,
                "direct": "O(N^2) FP64 sum excluding same-patch and near-singular pairs, plus the singular corrections"}
    # end to end: host buffers through the C ABI (copies in the timed region)
    xp = torch.from_numpy(x_h).pin_memory()
    yp = torch.empty_like(xp).pin_memory()
    k_e2e = max(1, min(args.steps, 500))
    px, py = G._dp(xp.numpy().view(np.float64)), G._dp(yp.numpy().view(np.float64))
    h = fm.handle
    for _ in range(3):
        L.ifgf2d_apply(h, px, py, 1)
    torch.cuda.synchronize()
    e2, e3 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e2.record(ext)
    for _ in range(k_e2e):
        rc = L.ifgf2d_apply(h, px, py, 1)
        assert rc == 0
    e3.record(ext)
    torch.cuda.synchronize()
    e2e_ms = e2.elapsed_time(e3) / k_e2e
    y_dev = y.cpu().numpy()
    assert np.allclose(yp.numpy(), y_dev, rtol=0, atol=1e-12 * np.abs(y_dev).max()), "e2e result differs"
    # per-phase timings (CUDA events between the phases, on the context's stream)
    phases = ["sing_correction", "intensities", "leaf_cones", "propagation", "near_interp"]
    acc = np.zeros(5)
    nrep = max(10, min(args.steps, 200))
    buf = (ctypes.c_double * 5)()
    for _ in range(nrep):
        rc = L.ifgf2d_apply_timed(fm.handle, x.data_ptr(), y.data_ptr(), 1, buf)
        assert rc == 0
        acc += np.array(buf[:])
    acc /= nrep
    acc_mixed = np.zeros(5)
    for _ in range(nrep):
        rc = L.ifgf2d_apply_timed(fm.handle, x.data_ptr(), y.data_ptr(), 2, buf)
        assert rc == 0
        acc_mixed += np.array(buf[:])
    acc_mixed /= nrep
    P = fm.Ps * fm.Pang
    nl = fm.nlevels
    # coefficient writes are bounded by the total cone count (a small term)
    model = phase_model(wc, N, P, ncones_leaf=wc["cones"], nparent=wc["cones"])
    dom = int(np.argmax(acc))
    dname = phases[dom]
    peaks = measured_peaks()
    hbm = peaks.get("hbm_gbs", 6800.0)
    fp64_peak = ctypes.c_double(0.0)
    L.ifgf2d_measure_fp64_peak(ctypes.byref(fp64_peak))
    bytes_d, flops_d = model[dname]
    achieved = bytes_d / (acc[dom] * 1e-3) / 1e9
    # DRAM bytes per launch of each phase from the committed ncu capture of this workload
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        try:
            traffic = json.load(open(tpath)).get("phases_fp64", {}).get(dname)
        except Exception:
            traffic = None
    roofline = {"bound": "hbm", "kernel": dname, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm, "traffic": traffic,
                "traffic_source": "profiles/traffic.json: ncu dram__bytes_read.sum + dram__bytes_write.sum of this phase's "
                                  "kernels in one FP64 apply of this workload (not measured in this run)",
                "peak_source": "measured" if "hbm_gbs" in peaks else "fallback",
                "fp64": {"achieved_tflops": flops_d / (acc[dom] * 1e-3) / 1e12, "peak_tflops": fp64_peak.value,
                         "frac": (flops_d / (acc[dom] * 1e-3) / 1e12) / max(fp64_peak.value, 1e-9),
                         "peak_source": "measured (ifgf2d_measure_fp64_peak)"},
                "phase_ms": dict(zip(phases, [float(v) for v in acc]))}
    # every phase against its own roof (FP64 pipe or HBM), weighted by its time
    per_phase = {}
    for i, ph in enumerate(phases):
        b_i, f_i = model[ph]
        t_i = acc[i] * 1e-3
        per_phase[ph] = max(b_i / t_i / 1e9 / hbm, f_i / t_i / 1e12 / max(fp64_peak.value, 1e-9))
    roofline["time_weighted"] = {"frac": float(sum(acc[i] * per_phase[ph] for i, ph in enumerate(phases)) / acc.sum()),
                                 "per_phase_frac": per_phase,
                                 "roofs": "each phase: max(HBM bytes / measured copy GB/s, FP64 flops / measured FP64 peak)"}
    # the fixed nominal weights of the work model: 60 flops per Hankel value, 20 per e^{ikr}/sqrt(r),
    # 8 per complex multiply-add; compulsory HBM bytes with complex128 = 16 B
    F_H, F_E = 60, 20
    sing_mv = wc["sing_entries"] + fm.num_patches_ * NP * NP
    nom_flops = (wc["near_pairs"] * (8 + F_H) + wc["leaf_evals"] * (8 + F_H) + wc["prop_evals"] * (8 * P + F_E)
                 + wc["interp_evals"] * (8 * P + F_E) + wc["cones"] * P * 2 * (fm.Ps + fm.Pang) * 4 + 8 * sing_mv)
    nom_bytes = N * (32 + 16 + 16) + 16 * wc["sing_entries"] + 2 * 16 * P * wc["cones"]
    t_mv = ms / args.steps * 1e-3
    roofline["nominal_model"] = {"flops_per_matvec": int(nom_flops), "bytes_per_matvec": int(nom_bytes),
                                 "tflops": nom_flops / t_mv / 1e12, "gbs": nom_bytes / t_mv / 1e9,
                                 "weights": {"hankel": F_H, "exp_over_sqrt": F_E, "complex_mac": 8}}
    # GMRES solve to 1e-6 (plane wave at angle 0), plain FP64 IFGF
    solve = None
    if not args.no_solve:
        b = -np.exp(1j * K_WAVE * fm.xs_)
        solve = {}
        fm.spectral_setup()
        for name, mixed, spec in (("plain_fp64", False, False), ("chosen_mixed", True, False), ("chosen_mixed_spectral", True, True)):
            times = []
            for _ in range(3):   # first call: Krylov workspace + graph capture; then warm solves
                t0 = time.perf_counter()
                if spec:
                    xs = fm.solve_flexible(b, "spectral", tol=1e-6, restart=300, max_iters=3000, mixed=mixed)
                else:
                    xs = fm.gmres(b, accelerated=True, tol=1e-6, restart=300, max_iters=3000, mixed=mixed)
                times.append(time.perf_counter() - t0)
            true_res = float(np.linalg.norm(fm.compute_Ax_acc(xs) - b) / np.linalg.norm(b))
            solve[name] = {"seconds": min(times[1:]), "seconds_first_call": times[0], "iters": fm.last_solve["iters"],
                           "fp64_refinement_passes": fm.last_solve.get("refinements", 0),
                           "converged": fm.last_solve["converged"], "true_rel_residual_fp64": true_res, "tol": 1e-6,
                           "restart": 300}
        solve["speedup_chosen_vs_plain"] = solve["plain_fp64"]["seconds"] / solve["chosen_mixed"]["seconds"]
        solve["speedup_spectral_vs_plain"] = solve["plain_fp64"]["seconds"] / solve["chosen_mixed_spectral"]["seconds"]
    # one apply = fused singular correction + intensities, leaf cones, nl - 3 propagation
    # levels, near field + interpolation
    launches_per_apply = 1 + 1 + (nl - 3) + 1
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded kite geometry, mt19937(0) density)",
        "config": {"workload": WORKLOAD, "N": N, "k": K_WAVE, "nlevels": nl, "patches": NPATCH, "Np": NP,
                   "Ps": fm.Ps, "Pang": fm.Pang, "parallelism": f"replicas x{world}",
                   "tuning": {"leaf_chunks_fp64": int(fm.tuning[0]), "leaf_chunks_c64": int(fm.tuning[1]),
                              "prop_cones_per_block_fp64": [int(v) for v in fm.tuning[2:2 + 24][3:nl]],
                              "prop_cones_per_block_c64": [int(v) for v in fm.tuning[2 + 24:][3:nl]]},
                   "l2": f"per-step streamed tables {wc['resident_bytes'] / 1e6:.0f} MB > 129 MB L2 (no flush)"},
        "e2e": {"value": world / (e2e_ms * 1e-3), "unit": UNIT, "h2d_bytes_per_step": 16 * N, "d2h_bytes_per_step": 16 * N,
                "ms_per_step": e2e_ms},
        "roofline": roofline,
        "clocks": clk.summary(),
        "gpu_launches": launches_per_apply * args.steps,
        "solve": solve,
        "chosen": {"form": "IFGF far field complex64 (FP32 arithmetic, FP64-computed tables), FP64 singular correction",
                   "value": world * args.steps / (ms_mixed * 1e-3), "unit": UNIT, "ms_per_step": ms_mixed / args.steps,
                   "rel_err_vs_fp64": mixed_err,
                   "phase_ms": dict(zip(phases, [float(v) for v in acc_mixed]))},
        "work": wc,
        "accuracy": accuracy,
    }
    if world > 1:   # the extra workloads are single-GPU measurements, reported at N = 1
        return out
    if not args.no_solve:
        out["config1"] = run_config1(G)
    if not args.no_batch:
        del fm
        torch.cuda.synchronize()
        out["batch"] = run_batch(G, k=args.batch_k, npatch=args.batch_patches, solve=not args.no_solve)
    if not args.no_large and not args.no_solve:
        out["large"] = run_large(G)
    if not args.no_obstacles and not args.no_solve:
        out["obstacles"] = run_obstacles()
    if not args.no_learned and not args.no_solve:
        out["preconditioned"] = run_preconditioned(G, cases=tuple((float(v), int(round(1.024 * float(v))))
                                                                  for v in args.precond_k.split(",") if v))
    return out


def run_preconditioned(G, cases=((2000.0, 2048), (8000.0, 8192))):
    """Right preconditioners on the kite, all solves to a 1e-6 FP64 true residual: plain FP64
    GMRES; FP64 refinement around complex64 GMRES ("mixed"); the same with flexible GMRES and the
    spectral preconditioner (inverse flat-boundary symbol along the curve), alone and corrected
    by the learned network trained on its errors; and the first network alone (trained on the
    errors of 2I).  Set-up-inclusive times add the constructor, precomps_and_setup and, for the
    spectral forms, the preconditioner's tables."""
    from ifgf2d_gb300.learned import PreconditionerNet, DEFAULT_WEIGHTS, SPECTRAL_WEIGHTS
    nets = {}
    for key, path in (("net", DEFAULT_WEIGHTS), ("spectral_net", SPECTRAL_WEIGHTS)):
        if os.path.exists(path):
            nets[key] = PreconditionerNet.load(path)
    res = {"weights": {k: os.path.relpath(p, ROOT) for k, p in (("net", DEFAULT_WEIGHTS), ("spectral_net", SPECTRAL_WEIGHTS))},
           "training": "pairs from plain FP64 GMRES iterates; k ~ U(50, 400), stars and kites, 10 points per wavelength",
           "spectral_scale": None}
    for k, npatch in cases:
        import torch
        t0 = time.perf_counter()
        fm = G.ForwardMap(DELTA, [G.Kite()], (), 1.0, k, Np=NP, patches_per_curve=npatch, formulation="combined")
        fm.precomps_and_setup(k, 0)
        torch.cuda.synchronize()
        setup_s = time.perf_counter() - t0
        t0 = time.perf_counter()
        fm.spectral_setup()
        spec_setup_s = time.perf_counter() - t0
        b = -np.exp(1j * k * fm.xs_)
        row = {"N": fm.total_num_unknowns_, "setup_s": setup_s, "spectral_setup_s": spec_setup_s}
        forms = [("plain_fp64", lambda: fm.gmres(b, tol=1e-6, restart=300, max_iters=3000)),
                 ("mixed", lambda: fm.gmres(b, tol=1e-6, restart=300, max_iters=3000, mixed=True)),
                 ("mixed_spectral", lambda: fm.solve_flexible(b, "spectral", tol=1e-6, restart=300, max_iters=3000, mixed=True))]
        if "spectral_net" in nets:
            forms.append(("mixed_spectral_net", lambda: fm.solve_flexible(b, "spectral+net", net=nets["spectral_net"], tol=1e-6,
                                                                          restart=300, max_iters=3000, mixed=True)))
        if "net" in nets:
            forms.append(("mixed_net", lambda: fm.solve_flexible(b, "net", net=nets["net"], tol=1e-6, restart=300, max_iters=3000,
                                                                 mixed=True)))
        for name, fn in forms:
            fn()
            torch.cuda.nvtx.range_push(f"{name}_k{int(k)}")   # profiler ranges (ncu --nvtx-include)
            t0 = time.perf_counter()
            x = fn()
            dt = time.perf_counter() - t0
            torch.cuda.nvtx.range_pop()
            tr = float(np.linalg.norm(fm.compute_Ax_acc(x) - b) / np.linalg.norm(b))
            row[name] = {"seconds": dt, "iters": fm.last_solve["iters"], "converged": fm.last_solve["converged"],
                         "fp64_refinement_passes": fm.last_solve.get("refinements", 0), "true_rel_residual_fp64": tr}
        plain = row["plain_fp64"]["seconds"]
        row["speedup_vs_plain"] = {n: plain / row[n]["seconds"] for n, _ in forms if n != "plain_fp64"}
        extra = {n: (spec_setup_s if "spectral" in n else 0.0) for n, _ in forms}
        row["with_setup"] = {n: setup_s + extra[n] + row[n]["seconds"] for n, _ in forms}
        row["with_setup"]["speedup_vs_plain"] = {n: row["with_setup"]["plain_fp64"] / row["with_setup"][n]
                                                 for n, _ in forms if n != "plain_fp64"}
        res[f"kite_k{int(k)}"] = row
        del fm
    res["spectral_scale"] = G._lib.SPECTRAL_DEFAULT_SCALE
    return res


def run_config1(G, repeats=5):
    """Unit circle, k = 10, 20 equal patches x 10 Fejer nodes (N = 200), combined field with
    eta = k, direct operator with the rectangular-polar singular weights, plane wave at angle 0,
    GMRES to 1e-10.  Device: precomputation + GMRES through the public API with host vectors
    (median of the repeats after the first).  CPU: the oracle's precomputation + Householder
    GMRES on one thread, as the reference runs (median of the second and third of three runs)."""
    from oracle import oracle as O
    O.build()
    k = 10.0
    fm = G.ForwardMap(DELTA, [G.Circle()], (), 1.0, k, Np=10, patches_per_curve=20, formulation="combined")
    b = -np.exp(1j * k * fm.xs_)
    dev = []
    for _ in range(repeats):
        t0 = time.perf_counter()
        x = fm.solve(b, k, accelerated=False, tol=1e-10)
        dev.append(time.perf_counter() - t0)
    it_dev = fm.last_solve["iters"]
    res_dev = float(np.linalg.norm(fm.compute_Ax_unacc(x) - b) / np.linalg.norm(b))
    om = O.OracleForwardMap([O.curve_circle()], 10, DELTA, 1.0, k, patches_per_curve=20, formulation="combined")
    cpu = []
    for _ in range(3):
        t0 = time.perf_counter()
        om.precompute(k)
        xo, info = om.solve(b, False, tol=1e-10)
        cpu.append(time.perf_counter() - t0)
    res_cpu = float(np.linalg.norm(om.compute_Ax_unacc(xo) - b) / np.linalg.norm(b))
    return {"workload": "unit circle k=10, 20 equal patches x 10 (N=200), combined field eta=k, direct operator, "
                        "plane wave at angle 0, GMRES to 1e-10",
            "N": fm.total_num_unknowns_,
            "device": {"seconds": float(np.median(dev[1:])), "seconds_first_call": dev[0], "iters": it_dev,
                       "true_rel_residual": res_dev, "path": "ifgf2d_precompute + ifgf2d_solve, host vectors"},
            "cpu_oracle_1_thread": {"seconds": float(np.median(cpu[1:])), "iters": int(info["iters"]),
                                    "true_rel_residual": res_cpu,
                                    "path": "oracle precompute + Householder GMRES (opGMRES.hpp:68-269)"},
            "rel_diff_solutions": float(np.linalg.norm(x - xo) / np.linalg.norm(xo))}


def run_large(G, k=8000.0, npatch=8192):
    """Kite k=8000, 8192 patches x 16 (N=131072), plane wave at angle 0: plain FP64 GMRES
    against FP64 refinement around complex64 inner solves, both to a 1e-6 FP64 residual."""
    import torch
    t0 = time.perf_counter()
    fm = G.ForwardMap(DELTA, [G.Kite()], (), 1.0, k, Np=NP, patches_per_curve=npatch, formulation="combined")
    fm.precomps_and_setup(k, 0)
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    fm.autotune()
    torch.cuda.synchronize()
    res = {"workload": f"kite k={k:g}, {npatch} patches x {NP} (N={fm.total_num_unknowns_}), combined field, plane wave",
           "N": fm.total_num_unknowns_, "nlevels": fm.nlevels, "setup_s": setup_s,
           "setup": "ForwardMap constructor (discretisation) + precomps_and_setup (RP weights, tree, plans, device tables)",
           "autotune_s": time.perf_counter() - t0}
    N = fm.total_num_unknowns_
    x = torch.from_numpy(G.seeded_density(N)).cuda()
    y = torch.empty_like(x)
    ext = torch.cuda.ExternalStream(fm.stream())
    for mixed in (False, True):
        for _ in range(3):
            fm.apply_device(x, y, mixed=mixed)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        for _ in range(10):
            fm.apply_device(x, y, mixed=mixed)
        e1.record(ext)
        torch.cuda.synchronize()
        res["apply_" + ("mixed" if mixed else "fp64") + "_ms"] = e0.elapsed_time(e1) / 10
    b = -np.exp(1j * k * fm.xs_)
    for name, mixed in (("plain_fp64", False), ("chosen_mixed", True)):
        times = []
        for _ in range(2):
            t0 = time.perf_counter()
            xs = fm.gmres(b, accelerated=True, tol=1e-6, restart=300, max_iters=3000, mixed=mixed)
            times.append(time.perf_counter() - t0)
        tr = float(np.linalg.norm(fm.compute_Ax_acc(xs) - b) / np.linalg.norm(b))
        res[name] = {"seconds": times[1], "seconds_first_call": times[0], "iters": fm.last_solve["iters"],
                     "fp64_refinement_passes": fm.last_solve.get("refinements", 0),
                     "converged": fm.last_solve["converged"], "true_rel_residual_fp64": tr}
    res["speedup_chosen_vs_plain"] = res["plain_fp64"]["seconds"] / res["chosen_mixed"]["seconds"]
    res["with_setup"] = {"plain_fp64_s": setup_s + res["plain_fp64"]["seconds"],
                         "chosen_mixed_s": setup_s + res["chosen_mixed"]["seconds"],
                         "speedup_chosen_vs_plain": (setup_s + res["plain_fp64"]["seconds"]) /
                                                    (setup_s + res["chosen_mixed"]["seconds"])}
    return res


def run_obstacles(n=256, plain_sample=256):
    """256 seeded star obstacles (k ~ U(10, 400), 10 points per wavelength, plane waves),
    each solved to a 1e-6 FP64 residual.  Chosen: host set-up of the next obstacles on 15
    host threads while 3 device threads run the obstacles' device work, each on its own
    context stream, complex64 inner solves.  Grouped: groups of 16 obstacles, each merged into
    one block-diagonal operator (one launch per phase, lock-step GMRES), 3 device threads.
    Plain: one obstacle after another, FP64 GMRES, on the first `plain_sample` obstacles."""
    from ifgf2d_gb300.scatterers import star_obstacles, solve_obstacles, solve_obstacles_grouped
    # groups of 16 obstacles on 3 device threads (the first call warms up), without and with the
    # spectral preconditioner
    res_g = {}
    for key, pc in (("grouped", None), ("grouped_spectral", "spectral")):
        for rep in range(2):
            obs = star_obstacles(n)
            t0 = time.perf_counter()
            solve_obstacles_grouped(obs, tol=1e-6, workers=15, mixed=True, chunk=16, device_threads=3, precond=pc)
            g = {"seconds": time.perf_counter() - t0}
        rg = [o.result for o in obs]
        g.update({"ms_per_obstacle": g["seconds"] / n * 1e3,
                  "all_converged": all(x["converged"] for x in rg),
                  "max_true_rel_residual_fp64": max(x["true_rel_residual"] for x in rg),
                  "grouped": int(sum(x.get("grouped", False) for x in rg)),
                  "iters_max": int(max(x["iters"] for x in rg)),
                  "iters_mean": float(np.mean([x["iters"] for x in rg])),
                  "form": "groups of 16 on 3 device threads: merged set-up, segmented lock-step GMRES, "
                          "complex64 inner solves, FP64 refinement" + (", flexible GMRES with the spectral preconditioner" if pc else "")})
        res_g[key] = g
    grouped = res_g["grouped"]
    obs = star_obstacles(n)
    t0 = time.perf_counter()
    solve_obstacles(obs, tol=1e-6, workers=15, mixed=True, device_threads=3)
    dt = time.perf_counter() - t0
    r = [o.result for o in obs]
    sub = star_obstacles(n)[:plain_sample]
    t0 = time.perf_counter()
    solve_obstacles(sub, tol=1e-6, workers=0, mixed=False)
    dtp = time.perf_counter() - t0
    rp = [o.result for o in sub]
    return {"workload": f"{n} star obstacles r = 1 + sum_m a_m cos mt + b_m sin mt (m <= 5, |a|,|b| < 0.05), "
                        "k ~ U(10, 400), N_i = 16 ceil(10 k L / 2 pi / 16), plane wave at a random angle; numpy default_rng(0)",
            "n": n, "unknowns_total": int(sum(o.npoints for o in obs)),
            "grouped": grouped,
            "grouped_spectral": res_g["grouped_spectral"],
            "chosen": {"seconds": dt, "ms_per_obstacle": dt / n * 1e3, "device_threads": 3,
                       "all_converged": all(x["converged"] for x in r),
                       "max_true_rel_residual_fp64": max(x["true_rel_residual"] for x in r),
                       "ifgf": int(sum(x["accelerated"] for x in r)), "direct": int(sum(not x["accelerated"] for x in r))},
            "plain": {"ms_per_obstacle": dtp / plain_sample * 1e3, "sample": f"the first {plain_sample} obstacles, one at a time",
                      "all_converged": all(x["converged"] for x in rp),
                      "max_true_rel_residual_fp64": max(x["true_rel_residual"] for x in rp)},
            "speedup_chosen_vs_plain_per_obstacle": (dtp / plain_sample) / (dt / n),
            "speedup_grouped_vs_plain_per_obstacle": (dtp / plain_sample) / (grouped["seconds"] / n),
            "speedup_grouped_spectral_vs_plain_per_obstacle": (dtp / plain_sample) / (res_g["grouped_spectral"]["seconds"] / n)}


def run_batch(G, k=2000.0, npatch=2048, nrhs=64, solve=True):
    """Many incidence angles, one operator: kite k=2000, 2048 patches x 16 (N=32768), plane
    waves at 2 pi j / nrhs.  The chosen form: batched complex64 applies inside FP64 iterative
    refinement (ifgf2d_solve_batch), against plain FP64 GMRES one right-hand side at a time."""
    import torch
    t0 = time.perf_counter()
    fm = G.ForwardMap(DELTA, [G.Kite()], (), 1.0, k, Np=NP, patches_per_curve=npatch, formulation="combined")
    fm.precomps_and_setup(k, 0)
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    N = fm.total_num_unknowns_
    ang = 2 * np.pi * np.arange(nrhs) / nrhs
    B = -np.exp(1j * k * (np.cos(ang)[None, :] * fm.xs_[:, None] + np.sin(ang)[None, :] * fm.ys_[:, None]))
    xt = torch.from_numpy(np.ascontiguousarray(B.T)).cuda()
    yt = torch.empty_like(xt)
    ext = torch.cuda.ExternalStream(fm.stream())
    res = {"workload": f"kite k={k:g}, {npatch} patches x {NP} (N={N}), combined field, {nrhs} plane waves at 2 pi j/{nrhs}",
           "N": N, "nrhs": nrhs, "nlevels": fm.nlevels, "setup_s": setup_s}
    # complex64 as configured; with every kernel on FP32 FMA; with the FMA propagation fed by TMA
    # bulk copies; with the leaf-cone sums, and leaf and propagation, on the tcgen05 tensor cores
    # (3xTF32); FP64
    default_tc = fm.batch_tensor_cores
    for name, mixed, tc in (("mixed", True, default_tc), ("mixed_fma", True, 0),
                            ("mixed_tma_propagation", True, fm.BATCH_BULK_PROPAGATION),
                            ("mixed_tcgen05_leaf_tma_propagation", True, fm.BATCH_TC_LEAF | fm.BATCH_BULK_PROPAGATION),
                            ("mixed_tcgen05_leaf", True, fm.BATCH_TC_LEAF),
                            ("mixed_tcgen05_leaf_propagation", True, fm.BATCH_TC_LEAF | fm.BATCH_TC_PROPAGATION),
                            ("fp64", False, default_tc)):
        fm.batch_tensor_cores = tc
        reps = 10 if mixed else 2
        for _ in range(2):
            fm.apply_batch_device(xt, yt, nrhs, mixed=mixed)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        for _ in range(reps):
            fm.apply_batch_device(xt, yt, nrhs, mixed=mixed)
        e1.record(ext)
        torch.cuda.synchronize()
        res["apply_" + name + "_us_per_rhs"] = e0.elapsed_time(e1) / reps / nrhs * 1e3
    fm.batch_tensor_cores = default_tc
    res["tcgen05_kernels"] = default_tc
    # per right-hand side: the complex64 batched apply against the FP64 one; the FP64 IFGF
    # against the FP64 O(N^2) direct sum for the first incidence angle
    fm.apply_batch_device(xt, yt, nrhs, mixed=False)
    torch.cuda.synchronize()   # the apply runs on the context's stream
    y64 = yt.cpu().numpy()
    fm.apply_batch_device(xt, yt, nrhs, mixed=True)
    torch.cuda.synchronize()
    y32 = yt.cpu().numpy()
    errs = np.linalg.norm(y32 - y64, axis=1) / np.linalg.norm(y64, axis=1)
    yd = fm.compute_Ax_unacc(B[:, 0])
    res["accuracy"] = {"mixed_rel_err_vs_fp64_per_rhs_max": float(errs.max()),
                       "mixed_rel_err_vs_fp64_per_rhs_median": float(np.median(errs)),
                       "ifgf_fp64_rel_err_vs_direct_rhs0": float(np.linalg.norm(y64[0] - yd) / np.linalg.norm(yd))}
    # one right-hand side through the single-vector path, for the per-RHS comparison
    y1 = torch.empty(N, dtype=torch.complex128, device="cuda")
    for mixed in (True, False):
        for _ in range(3):
            fm.apply_device(xt[0], y1, mixed=mixed)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        for _ in range(10):
            fm.apply_device(xt[0], y1, mixed=mixed)
        e1.record(ext)
        torch.cuda.synchronize()
        res["apply_" + ("mixed" if mixed else "fp64") + "_single_us"] = e0.elapsed_time(e1) / 10 * 1e3
    if not solve:
        return res
    # chosen: batched mixed solve (second call timed: the first allocates the Krylov basis)
    times = []
    for i in range(2):
        torch.cuda.nvtx.range_push(f"batch_solve_{i}")   # profiler ranges (ncu --nvtx-include)
        t0 = time.perf_counter()
        X = fm.gmres_batch(B, tol=1e-6, restart=300, max_iters=3000, mixed=True)
        times.append(time.perf_counter() - t0)
        torch.cuda.nvtx.range_pop()
    st = fm.last_solve
    R = fm.apply_batch(X) - B
    rr = np.linalg.norm(R, axis=0) / np.linalg.norm(B, axis=0)
    res["chosen_solve"] = {"form": "batched complex64 IFGF inner GMRES, FP64 refinement", "seconds": times[1],
                           "seconds_first_call": times[0], "ms_per_rhs": times[1] / nrhs * 1e3,
                           "iters_min": int(min(st["iters"])), "iters_max": int(max(st["iters"])),
                           "fp64_refinement_passes": st.get("refinements"),
                           "converged": bool(st["converged"]), "max_true_rel_residual_fp64": float(rr.max())}
    # chosen + spectral preconditioner: the same batch in flexible GMRES
    fm.spectral_setup()
    times = []
    for i in range(2):
        torch.cuda.nvtx.range_push(f"batch_solve_spectral_{i}")
        t0 = time.perf_counter()
        X = fm.gmres_batch(B, tol=1e-6, restart=300, max_iters=3000, mixed=True, precond="spectral")
        times.append(time.perf_counter() - t0)
        torch.cuda.nvtx.range_pop()
    st = fm.last_solve
    R = fm.apply_batch(X) - B
    rr = np.linalg.norm(R, axis=0) / np.linalg.norm(B, axis=0)
    res["chosen_solve_spectral"] = {"form": "batched flexible GMRES with the spectral preconditioner, complex64 inner solves, "
                                            "FP64 refinement", "seconds": times[1],
                                    "seconds_first_call": times[0], "ms_per_rhs": times[1] / nrhs * 1e3,
                                    "iters_min": int(min(st["iters"])), "iters_max": int(max(st["iters"])),
                                    "fp64_refinement_passes": st.get("refinements"),
                                    "converged": bool(st["converged"]), "max_true_rel_residual_fp64": float(rr.max())}
    # plain: FP64 GMRES, one right-hand side per call (as the reference solves), on two angles
    pt, its, pres = [], [], []
    for j in (0, nrhs // 4):
        t0 = time.perf_counter()
        x = fm.gmres(B[:, j], accelerated=True, tol=1e-6, restart=300, max_iters=3000)
        pt.append(time.perf_counter() - t0)
        its.append(fm.last_solve["iters"])
        pres.append(float(np.linalg.norm(fm.compute_Ax_acc(x) - B[:, j]) / np.linalg.norm(B[:, j])))
    res["plain_solve"] = {"form": "FP64 IFGF GMRES, one right-hand side per call", "ms_per_rhs": float(np.mean(pt[1:] or pt)) * 1e3,
                          "sample": "angles 0 and pi/2, the first call excluded when two ran", "iters": its,
                          "max_true_rel_residual_fp64": max(pres)}
    res["speedup_chosen_vs_plain_per_rhs"] = res["plain_solve"]["ms_per_rhs"] / res["chosen_solve"]["ms_per_rhs"]
    res["speedup_spectral_vs_plain_per_rhs"] = res["plain_solve"]["ms_per_rhs"] / res["chosen_solve_spectral"]["ms_per_rhs"]
    return res


def time_oracle(budget_s=12.0, max_steps=None, threads=None, check=None):
    """The CPU oracle (restatement of the reference path, which is single-threaded) on the same
    workload, on every host thread: one oracle context per thread, each running whole IFGF
    matvecs until the common deadline; the value is all threads' matvecs over the wall time.

    With `check` (the device's FP64 and complex64 applies of the seeded density), the oracle's
    FP64 direct forward map of the same density -- singular corrections plus the O(N^2) sum
    with the same exclusions plus the jump term, rows split over the threads' contexts -- and
    its IFGF apply are compared with them."""
    import threading
    from concurrent.futures import ThreadPoolExecutor
    from oracle import oracle as O
    O.build()
    nt = threads or max(1, min(32, os.cpu_count() or 1))

    def make():
        om = O.OracleForwardMap([O.curve_kite()], NP, DELTA, 1.0, K_WAVE, patches_per_curve=NPATCH, formulation="combined")
        om.precompute(K_WAVE)
        # same tree depth rule as the product: deepest nlevels passing the neighbourhood check
        for nl in range(16, 2, -1):
            try:
                om.setup_ifgf(K_WAVE, nl)
                return om, nl
            except RuntimeError:
                continue
        raise RuntimeError("oracle: no valid tree depth")

    with ThreadPoolExecutor(nt) as ex:
        ctxs = list(ex.map(lambda _: make(), range(nt)))
    d = O.seeded_density(ctxs[0][0].N)
    counts = [0] * nt
    ends = [0.0] * nt
    per_thread_cap = None if max_steps is None else max(1, -(-max_steps // nt))
    t_start = time.perf_counter()
    deadline = t_start + budget_s

    def run(i):
        om = ctxs[i][0]
        while True:
            om.compute_Ax_acc(d)
            counts[i] += 1
            ends[i] = time.perf_counter()
            if ends[i] >= deadline or (per_thread_cap is not None and counts[i] >= per_thread_cap):
                return

    ths = [threading.Thread(target=run, args=(i,)) for i in range(nt)]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    wall = max(ends) - t_start
    steps = sum(counts)
    out = {"value": steps / wall, "unit": UNIT, "cores": nt, "kind": "port",
           "sample": f"{steps} full IFGF matvecs of the same workload (nlevels {ctxs[0][1]}) on {nt} threads, "
                     f"one oracle context each, {wall:.1f} s wall"}
    if check:
        dens = check["density"]
        om0 = ctxs[0][0]
        w = om0.point_weights()[0]
        n = om0.N
        t0 = time.perf_counter()
        with ThreadPoolExecutor(nt) as ex:
            bounds = [(n * i // nt, n * (i + 1) // nt) for i in range(nt)]
            parts = list(ex.map(lambda i: ctxs[i][0].direct_excluded(dens * w, bounds[i]), range(nt)))
        y_dir = om0.sing_near_sing(dens) + np.concatenate(parts) + 0.5 * dens   # combined field: + 1/2 I
        y_ifgf = om0.compute_Ax_acc(dens)

        def rel(a, b):
            return float(np.linalg.norm(a - b) / np.linalg.norm(b))

        out["check"] = {"ifgf_fp64_rel_err_vs_oracle_direct": rel(check["y_fp64"], y_dir),
                        "ifgf_mixed_rel_err_vs_oracle_direct": rel(check["y_mixed"], y_dir),
                        "ifgf_fp64_rel_err_vs_oracle_ifgf": rel(check["y_fp64"], y_ifgf),
                        "oracle_ifgf_rel_err_vs_oracle_direct": rel(y_ifgf, y_dir),
                        "oracle_s": time.perf_counter() - t0,
                        "direct": "the oracle's FP64 O(N^2) direct map: singular corrections, the sum excluding "
                                  "same-patch and near-singular pairs, the jump term"}
    return out


def run_reference(args, rank, world):
    if rank != 0:
        return None
    r = time_oracle(budget_s=float(os.environ.get("IFGF2D_REF_BUDGET_S", "30")),
                    max_steps=max(1, args.steps))
    return {
        "metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded kite geometry, mt19937(0) density)", "impl": "reference",
        "config": {"workload": WORKLOAD, "parallelism": "host cores"},
        "cpu_baseline": r,
        "e2e": {"value": r["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    args = parse()
    rank, local_rank, world = dist_env()
    if args.impl == "reference":
        out = run_reference(args, rank, world)
        if out is not None:
            print(json.dumps(out), flush=True)
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    out = run_ours(args, rank, local_rank, world)
    if rank == 0:
        if world == 1 and not args.no_cpu_baseline:
            out["cpu_baseline"] = time_oracle(budget_s=12.0, check=CHECK or None)
            one = time_oracle(budget_s=6.0, threads=1)
            out["cpu_baseline"]["single_thread"] = {"value": one["value"], "unit": one["unit"], "sample": one["sample"]}
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
