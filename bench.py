"""Benchmark of the GB300 second-order evolver.

A "step" evolves every (k1,k2,k3) triplet of the workload once and fills the
ppt2->sources layout.  The default workload is the plain-vs-reference
configuration of the benchmark set: flat LCDM, k1,k2 on 25 log points in
[1e-5, 0.1]/Mpc, 15 k3 per pair (4875 triplets), T+E sources with l_max = 12,
m in {0,1,2}, rtol 1e-4, 200 source times from 200 Mpc to tau0.  Inputs are
synthetic: the background/recombination and first-order tables come from this
project's own provider (the CLASS tables the reference would use are not
available).

  value        triplets/s of the mixed form (FP64 RHS/residual/error control,
               FP32 banded LU of the per-m iteration-matrix blocks), tables
               resident in HBM, CUDA events around each persistent-kernel
               launch; L2 is flushed between steps.
  plain_fp64   the same for the plain FP64 form (FP64 banded LU), for the
               mixed-vs-plain ratio the metric asks for.
  e2e          triplets/s through song2_gpu_evolve (the drop-in C ABI): host
               tables uploaded and the host ppt2->sources slabs filled inside
               the timed region.
  cpu_baseline the CPU restatement (oracle/) on this machine's host cores, on a
               bounded sample of the same triplets.

--impl reference runs the reference arm: the reference (coccoinomane/song)
cannot be built (its CLASS submodule is empty), so the arm times the CPU
restatement of its algorithm with all host threads.
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "2nd-order k-triplets/s at rtol 1e-4: mixed+batched vs plain FP64 GPU; err vs FP64"
WORKLOAD = 2
# FP64 work of the mixed-form evolver per NDF step (ncu, reduced config 2) and the
# FP64 issue rate of a GB300 SM (DFMA probe, song_gb300/csrc/probe_fp64.cu)
FP64_FLOPS_PER_STEP = 47.0e3
FP64_WARP_INSTR_PER_STEP = 2.74e3
FP64_WARP_INSTR_PER_SM_CYCLE = 0.0526


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", type=int, default=WORKLOAD)
    ap.add_argument("--cpu-sample-s", type=float, default=15.0)
    ap.add_argument("--accuracy-sample", type=int, default=32,
                    help="triplets checked against the FP64 oracle at rtol 1e-8 (0: skip)")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--k-size", type=int, default=None, help="override the k grid size (small profiling cases)")
    ap.add_argument("--k3-size", type=int, default=None, help="override the k3 grid size (small profiling cases)")
    ap.add_argument("--rsa", type=int, default=0, choices=[0, 1, 2],
                    help="radiation-streaming approximation of both arms: 0 none (default), 1 MD, 2 MD with reio")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.path = os.path.join(ROOT, "gpurun_out", f"clocks_gpu{gpu}.csv")

    def __enter__(self):
        os.makedirs(os.path.dirname(self.path), exist_ok=True)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={q}", "--format=csv",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, ValueError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        try:
            lines = [l.strip() for l in open(self.path) if l.strip() and not l.startswith("index")]
        except OSError:
            return None
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in lines:
            parts = [p.strip() for p in l.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1].split()[0]))
                smax = float(parts[2].split()[0])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return {}


def build_problem(cfg, overrides):
    from song_gb300.problem import config_problem
    p = config_problem(cfg, **overrides)
    p.first_order_gpu()          # first-order tables from the GPU first-order mode (untimed set-up)
    return p


def table_bytes(p):
    return int(p.bg.nbytes * 2 + p.fo.nbytes * 2 + p.k.nbytes + p.k3.nbytes + p.tau.nbytes + p.k3_size.nbytes)


def algorithmic_bytes(p):
    """Bytes a step must move: the two first-order rows of every triplet's (k1,k2)
    pair over its time range (read once per pair and reused from L2 by the other k3
    of the pair), the background table, and the source writes."""
    per_pair_rows = 2 * p.fo.shape[1] * p.fo.shape[2] * 8 * 2   # values + spline d2 of two k rows
    n = len(p.k)
    n_pairs = n * (n + 1) // 2
    return int(n_pairs * per_pair_rows + 2 * p.bg.nbytes + p.tp2_size * p.per_type * 8)


def flush_l2(torch, buf):
    buf.zero_()


def run_device(lib, p, precision, steps, warmup, torch, rank, world):
    from song_gb300 import capi
    import torch.distributed as dist
    c = C.c_void_p()
    err = capi.errbuf()
    if lib.song2_ctx_create(C.byref(p.spec), C.byref(p.tables), precision, C.byref(c), err):
        raise RuntimeError(err.value.decode())
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    try:
        for _ in range(warmup):
            if lib.song2_ctx_run(c, None, err):
                raise RuntimeError(err.value.decode())
        ms = []
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        for _ in range(steps):
            flush_l2(torch, flush)
            torch.cuda.synchronize()
            if lib.song2_ctx_run(c, None, err):      # CUDA events on the launching stream inside
                raise RuntimeError(err.value.decode())
            ms.append(lib.song2_ctx_last_kernel_ms(c))
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        stats = (capi.TripletStats * p.n_triplets)()
        src = np.zeros(p.tp2_size * p.per_type)
        lib.song2_ctx_download(c, capi.dptr(src), stats, err)
        st = np.frombuffer(stats, dtype=capi.STATS_DTYPE).copy()
        launches = lib.song2_ctx_last_launches(c) * steps
    finally:
        lib.song2_ctx_destroy(c)
    return ms, st, src, launches


def run_e2e(lib, p, precision, steps, warmup):
    """song2_gpu_evolve with host tables and host nested slabs, wall time on the host
    around a synchronous call (the call returns after its D2H copies)."""
    from song_gb300 import capi
    n = len(p.k)
    keep = []
    tp_level = (C.POINTER(C.POINTER(C.POINTER(C.c_double))) * p.tp2_size)()
    d2h = 0
    for tp in range(p.tp2_size):
        k1_level = (C.POINTER(C.POINTER(C.c_double)) * n)()
        for i1 in range(n):
            k2_level = (C.POINTER(C.c_double) * (i1 + 1))()
            for i2 in range(i1 + 1):
                buf = np.zeros(len(p.tau) * int(p.k3_size[i1 * n + i2]))
                d2h += buf.nbytes
                keep.append(buf)
                k2_level[i2] = capi.dptr(buf)
            keep.append(k2_level)
            k1_level[i1] = k2_level
        keep.append(k1_level)
        tp_level[tp] = k1_level
    st = (capi.TripletStats * p.n_triplets)()
    err = capi.errbuf()
    times = []
    for i in range(warmup + steps):
        t0 = time.perf_counter()
        if lib.song2_gpu_evolve(C.byref(p.spec), C.byref(p.tables), precision, C.cast(tp_level, C.c_void_p), st,
                                err):
            raise RuntimeError(err.value.decode())
        if i >= warmup:
            times.append(time.perf_counter() - t0)
    return times, table_bytes(p), d2h


def cpu_baseline(p, budget_s, threads):
    """The oracle on a bounded, evenly spread sample of the same triplets."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    order = np.arange(p.n_triplets)
    # calibrate with a small sample, then size the sample to the budget
    n0 = min(p.n_triplets, max(threads, 8))
    pick = order[:: max(1, p.n_triplets // n0)][:n0]
    t0 = time.perf_counter()
    oracle.evolve(p, nthreads=threads, items=pick)
    dt = time.perf_counter() - t0
    per = dt / len(pick)
    n1 = int(min(p.n_triplets, max(len(pick), budget_s / max(per, 1e-6))))
    pick = order[:: max(1, p.n_triplets // n1)][:n1]
    t0 = time.perf_counter()
    oracle.evolve(p, nthreads=threads, items=pick)
    dt = time.perf_counter() - t0
    return len(pick) / dt, len(pick), dt


def accuracy_sample(p, results, n, threads, rtol=1e-8, floor=1e-10):
    """Max relative error of GPU sources against the FP64 oracle at rtol = 1e-8 on an
    evenly spread sample of n triplets: per (source type, triplet) max_tau |S - S_ref| /
    max_tau |S_ref|, the denominator floored at `floor` times the triplet's largest
    source (odd-m sources vanish by symmetry when k1 = k2)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    work = p.work_order()
    pick = list(range(0, len(work), max(1, len(work) // n)))[:n]
    ref, _ = oracle.evolve(p, nthreads=threads, items=np.array(pick), rtol=rtol)
    b = ref.reshape(p.tp2_size, p.per_type)
    out = {}
    for name, flat in results.items():
        a = flat.reshape(p.tp2_size, p.per_type)
        worst = 0.0
        for it in pick:
            i1, i2, i3 = work[it]
            ta, tb = p.triplet_view(a, i1, i2, i3), p.triplet_view(b, i1, i2, i3)
            den = np.max(np.abs(tb), axis=1)
            den = np.maximum(den, floor * max(den.max(), 1e-300))
            worst = max(worst, float(np.max(np.max(np.abs(ta - tb), axis=1) / den)))
        out[name] = worst
    return out, len(pick)


def main():
    args = parse()
    rank, world, local = dist_env()
    cfg_name = None
    from song_gb300.problem import CONFIGS
    cfg = dict(CONFIGS[args.config])
    overrides = {}
    if args.k_size:
        overrides["k_size"] = cfg["k_size"] = args.k_size
    if args.k3_size:
        overrides["k3_size"] = cfg["k3_size"] = args.k3_size
    cfg_name = cfg["name"] + ("" if not overrides else "_reduced")
    if args.rsa:
        overrides["radiation_streaming_approximation"] = args.rsa
        cfg_name += "_rsa%d" % args.rsa
    config = {"workload": cfg_name, "triplets_per_gpu": None, "k_min": cfg["k_min"], "k_max": cfg["k_max"],
              "k_size": cfg["k_size"], "k3_size": cfg["k3_size"], "l_max": cfg["l_max"], "m": list(cfg["m"]),
              "rtol": cfg["rtol"], "tau_size": cfg["tau_size"], "sources": cfg["sources"],
              "l2": "flushed between steps (256 MiB write)", "rsa": args.rsa}

    if args.impl == "reference":
        if rank != 0:
            return 0
        from song_gb300 import build
        build.build()
        from song_gb300.problem import config_problem
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        p = config_problem(args.config, **overrides)
        p.set_first_order(oracle.first_order(p, nthreads=os.cpu_count()))
        threads = os.cpu_count()
        vals = []
        for i in range(args.warmup + args.steps):
            v, n, dt = cpu_baseline(p, args.cpu_sample_s / max(1, args.steps), threads)
            if i >= args.warmup:
                vals.append((v, n, dt))
        v = statistics.median([x[0] for x in vals])
        config["triplets_per_gpu"] = p.n_triplets
        line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "triplets/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * p.n_triplets / v,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (own background/recombination and first-order provider)", "config": config,
                "cpu_baseline": {"value": v, "unit": "triplets/s", "cores": threads, "kind": "port",
                                 "sample": f"{vals[-1][1]} triplets spread over the {p.n_triplets}-triplet "
                                           f"workload per step ({vals[-1][2]:.1f} s)"},
                "e2e": {"value": v, "unit": "triplets/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "note": "reference (coccoinomane/song) does not build: its CLASS submodule class.git is empty; "
                        "this arm times the CPU restatement of its algorithm (oracle/) with all host threads"}
        print(json.dumps(line), flush=True)
        return 0

    import torch
    import torch.distributed as dist
    if world > 1:
        dist.init_process_group("nccl", init_method="env://")
        torch.cuda.set_device(local)
    else:
        torch.cuda.set_device(0)
    from song_gb300 import build, capi
    if rank == 0:
        build.build()
    if world > 1:
        dist.barrier()
    lib = capi.load()
    p = build_problem(args.config, overrides)
    n_trip = p.n_triplets
    config["triplets_per_gpu"] = n_trip

    with Clocks(local) as clk:
        ms_mixed, st_mixed, src_mixed, launches = run_device(lib, p, capi.SONG2_PREC_MIXED, args.steps,
                                                             args.warmup, torch, rank, world)
    clocks = clk.summary()
    ms_plain = None
    if not args.no_plain:
        ms_plain, st_plain, src_plain, _ = run_device(lib, p, capi.SONG2_PREC_FP64, max(1, args.steps),
                                                      max(1, min(args.warmup, 1)), torch, rank, world)
    # max over ranks of the timed device time
    t_mixed = sum(ms_mixed) / 1e3
    tt = torch.tensor([t_mixed], dtype=torch.float64, device="cuda")
    if world > 1:
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    t_mixed = float(tt.item())
    value = world * n_trip * args.steps / t_mixed

    e2e = None
    if not args.no_e2e:
        times, h2d, d2h = run_e2e(lib, p, capi.SONG2_PREC_MIXED, max(1, args.steps), 1)
        te = torch.tensor([sum(times)], dtype=torch.float64, device="cuda")
        if world > 1:
            dist.all_reduce(te, op=dist.ReduceOp.MAX)
        e2e = {"value": world * n_trip * len(times) / float(te.item()), "unit": "triplets/s",
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}

    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return 0

    peaks = measured_peaks()
    ms_step = 1e3 * t_mixed / args.steps
    alg = algorithmic_bytes(p)
    hbm_peak = peaks.get("hbm_gbs")
    achieved = alg / (ms_step / 1e3) / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": (achieved / hbm_peak) if hbm_peak else None, "traffic": None,
                "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if hbm_peak else "fallback 6800",
                "note": "the evolver is bound by the FP64 pipe (RHS, residual, error control), not by HBM; "
                        "bytes = first-order rows of every (k1,k2) pair + background + source writes"}
    steps_tot = st_mixed["n_steps"].sum()
    # FP64 pipe: algorithmic FP64 work per NDF step (ncu counters of this kernel on
    # the reduced config-2 case) and the SM's FP64 issue rate (the DFMA probe in
    # song_gb300/csrc/probe_fp64.cu); the run supplies the step count and the time
    sm_mhz = (clocks or {}).get("sm_mhz") or 2070.0
    nsm = torch.cuda.get_device_properties(0).multi_processor_count
    fp64_flops = steps_tot * FP64_FLOPS_PER_STEP / (ms_step / 1e3)
    fp64_peak = FP64_WARP_INSTR_PER_SM_CYCLE * 32 * 2 * sm_mhz * 1e6 * nsm
    fp64_slots = steps_tot * FP64_WARP_INSTR_PER_STEP / (ms_step / 1e3)
    slot_peak = FP64_WARP_INSTR_PER_SM_CYCLE * sm_mhz * 1e6 * nsm
    roofline_fp64 = {"bound": "fp64", "achieved": fp64_flops / 1e12, "peak": fp64_peak / 1e12, "unit": "TFLOP/s",
                     "frac": fp64_flops / fp64_peak, "issue_slots_frac": fp64_slots / slot_peak,
                     "note": "FP64 flops (FMA = 2) per NDF step from the ncu counters of this kernel; peak from "
                             "the DFMA probe (one FP64 warp instruction per ~19 SM cycles, any lane count); "
                             "issue_slots_frac counts FP64 warp instructions against that rate"}
    line = {"metric": METRIC, "value": value, "unit": "triplets/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64 (FP32 banded LU)",
            "data": "synthetic (own background/recombination and first-order provider)", "config": config,
            "gpu_launches": int(launches), "clocks": clocks, "roofline": roofline, "roofline_fp64": roofline_fp64,
            "e2e": e2e,
            "status_ok": bool(np.all(st_mixed["status"] == 0)),
            "counters": {"ndf_steps": int(steps_tot), "rhs": int(st_mixed["n_rhs"].sum()),
                         "jacobians": int(st_mixed["n_jac"].sum()), "lu": int(st_mixed["n_lu"].sum())}}
    if ms_plain is not None:
        t_plain = sum(ms_plain) / 1e3
        v_plain = n_trip * len(ms_plain) / t_plain
        line["plain_fp64"] = {"value": world * v_plain, "unit": "triplets/s", "ms_per_step": 1e3 * t_plain / len(ms_plain),
                              "status_ok": bool(np.all(st_plain["status"] == 0))}
        line["mixed_over_plain"] = value / (world * v_plain)
        from song_gb300.problem import source_errors  # noqa: F401
        a = src_mixed.reshape(p.tp2_size, p.per_type)
        b = src_plain.reshape(p.tp2_size, p.per_type)
        den = np.max(np.abs(b)) + 1e-300
        line["mixed_vs_plain_max_abs_over_max"] = float(np.max(np.abs(a - b)) / den)
    if rank == 0 and world == 1:
        # the CPU leg: the oracle timed on a bounded sample, and used as the checker
        # of the GPU sources against its FP64 run at rtol 1e-8
        try:
            v, n, dt = cpu_baseline(p, args.cpu_sample_s, os.cpu_count())
            line["cpu_baseline"] = {"value": v, "unit": "triplets/s", "cores": os.cpu_count(), "kind": "port",
                                    "sample": f"{n} triplets spread over the {n_trip}-triplet workload ({dt:.1f} s)"}
        except Exception as e:  # noqa: BLE001
            line["cpu_baseline"] = {"value": None, "error": str(e)[:200]}
        if args.accuracy_sample > 0:
            try:
                res = {"mixed": src_mixed}
                if ms_plain is not None:
                    res["plain_fp64"] = src_plain
                errs, npick = accuracy_sample(p, res, args.accuracy_sample, os.cpu_count())
                line["err_vs_fp64_oracle"] = dict(errs, sample_triplets=npick, oracle_rtol=1e-8,
                                                  metric="max over source types and sampled triplets of "
                                                         "max_tau|S - S_ref| / max_tau|S_ref|")
            except Exception as e:  # noqa: BLE001
                line["err_vs_fp64_oracle"] = {"error": str(e)[:200]}
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
