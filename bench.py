"""Benchmark of the GB300 second-order evolver.

A "step" is one pass of the evolver over one part of the workload.  The default
workload is the uneven batch of the benchmark set (config 4): flat LCDM, k1, k2
on 50 log points in [1e-5, 0.3]/Mpc, 24 k3 per pair (30,600 triplets), T+E+B
sources, l_max = min(40, 8 + ceil(k tau_rec / 2)) and m_max drawn from {0, 2, 4}
per triplet (96 hierarchy classes, 32 to 744 equations), rtol 1e-4, 200 source
times from 200 Mpc to tau0.  The triplets are dealt into K = --steps
cost-balanced parts (round-robin over each launch group's cost-sorted work
list), so the K timed steps evolve every triplet exactly once.  Consecutive
parts run on --contexts contexts and streams (song2_ctx_enqueue_part), so that
the last triplets of one part share the GPU with the next parts.
Inputs are synthetic: the background/recombination and first-order tables come
from this project's own provider (the CLASS tables the reference would use are
not available).

  value        triplets/s of the mixed form (FP64 right-hand side, Newton residual
               and error control; FP32 factorisation of the structured iteration
               matrix), tables resident in HBM, one pair of CUDA events around
               all K parts' launches; L2 is not flushed between steps because a
               step's working set exceeds it.
  plain_fp64   the plain FP64 form on the first --plain-parts parts, and the
               mixed form's time on the same parts (mixed_over_plain).
  e2e          triplets/s through song2_gpu_evolve (the drop-in C ABI) over the
               whole workload: host tables uploaded and the host ppt2->sources
               slabs filled inside the timed region.
  cpu_baseline the CPU restatement (oracle/) on this machine's host cores, on a
               bounded cost-stratified sample of the same triplets.
  contract     the mixed form at rtol 1e-6, where every sampled source meets
               the 1e-4 bound: throughput on the first --contract-parts parts
               and the error on the accuracy sample.
  transfer2    the line-of-sight integral (transfer2) of this run's sources on
               the device: transfer functions/s, the projection-table build, the
               CPU restatement on the heaviest pairs as baseline and parity check;
               inside it, bispectra: the intrinsic bispectrum (bispectra2) of
               those transfers still in HBM (T and E, synthetic first-order
               transfers), and the CPU restatement against the GPU on the same
               inputs with the l list cut to --bi-cpu-l multipoles.
  err_vs_fp64_oracle
               per (source type, triplet) max_tau |S - S_ref| / max_tau |S_ref| of
               the GPU sources against the oracle at rtol 1e-8, on triplets spread
               over every hierarchy size and m_max; computed in a spawned CPU
               process while the GPU arms run.

--impl reference runs the reference arm: the reference (coccoinomane/song)
cannot be built (its CLASS submodule is empty), so the arm times the CPU
restatement of its algorithm with all host threads, building its inputs with
the oracle library alone (no product library is loaded).  Each of its steps is
a cost-stratified sample of the workload; ms_per_step is the measured wall time
of a step.
"""
import argparse
import ctypes as C
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "2nd-order k-triplets/s at rtol 1e-4: mixed+batched vs plain FP64 GPU; err vs FP64"
WORKLOAD = 4
ERR_BOUND = 1e-4
# the rtol at which every sampled config-4 source meets ERR_BOUND against the
# rtol-1e-8 oracle (the global error of an rtol-1e-4 integration, GPU or CPU,
# is about 1.7e-3 on the squeezed triplets)
CONTRACT_RTOL = 1e-6
CONTRACT_PARTS = 20
# line-of-sight leg: the l sampling of the reference's precision presets
# (pre/*lmax2000.pre: l_max_scalars 2000, l_logstep 1.25, l_linstep 36)
LOS_L = (2000, 1.25, 36)
# Work of the mixed-form evolver per NDF step and DRAM traffic per triplet, from
# the ncu counters of both launch groups of the reduced config-4 case
# (python -m song_gb300.cases evolver --k-size 6: 504 triplets, 3.95 M NDF steps;
# FP64 flops = 2 DFMA + DMUL + DADD thread instructions, FP32 likewise), and the
# FP64 issue rate of a GB300 SM (one FP64 warp instruction per ~19 SM cycles
# whatever the number of active lanes; DFMA probe)
FP64_FLOPS_PER_STEP = 46.3e3
FP32_FLOPS_PER_STEP = 45.3e3
FP64_WARP_INSTR_PER_STEP = 1.73e3
FP64_WARP_INSTR_PER_SM_CYCLE = 0.0526
DRAM_BYTES_PER_TRIPLET = 10.8e6


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", type=int, default=WORKLOAD)
    ap.add_argument("--parts", type=int, default=0, help="parts of the workload (default: --steps)")
    ap.add_argument("--cpu-sample", type=int, default=256,
                    help="triplets of the CPU-baseline sample (every n/N-th of the cost-sorted workload)")
    ap.add_argument("--ref-step-items", type=int, default=64, help="triplets per reference-arm step")
    ap.add_argument("--accuracy-sample", type=int, default=16,
                    help="triplets checked against the FP64 oracle at rtol 1e-8 (0: skip)")
    ap.add_argument("--plain-parts", type=int, default=0, help="parts timed in plain FP64 (default: steps/4)")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--autotune-sample", type=int, default=256,
                    help="triplets the autotuner times its launch candidates on (0: default launch)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--contexts", type=int, default=4, help="contexts (and streams) the parts alternate over")
    ap.add_argument("--contract-parts", type=int, default=2,
                    help="parts (of 20) timed at the contract rtol (0: skip the contract leg)")
    ap.add_argument("--no-los", action="store_true", help="skip the line-of-sight (transfer2) leg")
    ap.add_argument("--los-reps", type=int, default=3)
    ap.add_argument("--los-cpu-share", type=float, default=0.05,
                    help="share of the transfer k units the CPU baseline of the line of sight runs")
    ap.add_argument("--no-bispectra", action="store_true", help="skip the intrinsic bispectrum leg")
    ap.add_argument("--bi-cpu-l", type=int, default=3,
                    help="multipoles (a prefix of the l list) of the bispectrum's CPU sample")
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
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region
    (written to a temporary file)."""

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        fd, self.path = tempfile.mkstemp(prefix=f"song2_clocks_gpu{gpu}_", suffix=".csv")
        os.close(fd)

    def __enter__(self):
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
        finally:
            try:
                os.unlink(self.path)
            except OSError:
                pass
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


def workload_overrides(args, cfg):
    overrides = {}
    if args.k_size:
        overrides["k_size"] = cfg["k_size"] = args.k_size
    if args.k3_size:
        overrides["k3_size"] = cfg["k3_size"] = args.k3_size
    name = cfg["name"] + ("" if not overrides else "_reduced")
    if args.rsa:
        overrides["radiation_streaming_approximation"] = args.rsa
        name += "_rsa%d" % args.rsa
    return overrides, name


def table_bytes(p):
    return int(p.bg.nbytes * 2 + p.fo.nbytes * 2 + p.k.nbytes + p.k3.nbytes + p.tau.nbytes + p.k3_size.nbytes)


def algorithmic_bytes(p):
    """Bytes a full pass must move: the two first-order rows of every (k1,k2) pair
    over the table's time range (values and spline coefficients, read once per pair
    and reused from L2 by the pair's other k3), the background table, and the source
    writes."""
    per_pair_rows = 2 * p.fo.shape[1] * p.fo.shape[2] * 8 * 2
    n = len(p.k)
    n_pairs = n * (n + 1) // 2
    return int(n_pairs * per_pair_rows + 2 * p.bg.nbytes + p.tp2_size * p.per_type * 8)


# ---------------------------------------------------------------- workload bookkeeping

def pair_order_classes(p):
    """Class (l_max, m_max) of every triplet in work order, or None for uniform runs."""
    if p.classes is None:
        return None
    n = len(p.k)
    start, off = {}, 0
    for i1 in range(n):
        for i2 in range(i1 + 1):
            start[(i1, i2)] = off
            off += int(p.k3_size[i1 * n + i2])
    out = []
    for (i1, i2, i3) in p.work_order():
        out.append(p.classes[int(p.triplet_class[start[(i1, i2)] + i3])])
    return out


def cost_order(p):
    """Work-order indices sorted by decreasing cost estimate (the GPU work list's
    order: max(k1, k2, k3), times (l_max + 1)(m_max + 1) for hierarchy classes)."""
    work = p.work_order()
    cls = pair_order_classes(p)
    n = len(p.k)
    kk = np.empty(len(work))
    off = {}
    acc = 0
    for i1 in range(n):
        for i2 in range(i1 + 1):
            off[(i1, i2)] = acc
            acc += int(p.k3_size[i1 * n + i2])
    for t, (i1, i2, i3) in enumerate(work):
        kk[t] = max(p.k[i1], p.k[i2], p.k3[off[(i1, i2)] + i3])
        if cls is not None:
            kk[t] *= (cls[t][0] + 1.0) * (cls[t][1] + 1.0)
    return np.argsort(-kk, kind="stable"), kk


def triplet_entries(p, items):
    """Flat indices (within one source type) of every (tau) entry of the given
    work-order triplets: array [len(items), tau_size]."""
    work = p.work_order()
    n = len(p.k)
    rows = []
    ntau = len(p.tau)
    for it in items:
        i1, i2, i3 = work[int(it)]
        nk3 = int(p.k3_size[i1 * n + i2])
        off = p.pair_offset(i1, i2)
        rows.append(off + i3 + nk3 * np.arange(ntau))
    return np.array(rows, dtype=np.int64)


def source_error(p, test, ref, items, floor=1e-10):
    """max over (source type, triplet) of max_tau |S - S_ref| / max_tau |S_ref| (the
    denominator floored at `floor` times the triplet's largest source: odd-m sources
    vanish by symmetry when k1 = k2) and the worst (source type, work-order index)."""
    a = test.reshape(p.tp2_size, p.per_type)
    b = ref.reshape(p.tp2_size, p.per_type)
    idx = triplet_entries(p, items)
    ta, tb = a[:, idx], b[:, idx]                     # [tp, triplet, tau]
    den = np.max(np.abs(tb), axis=2)
    den = np.maximum(den, floor * np.maximum(den.max(axis=0, keepdims=True), 1e-300))
    e = np.max(np.abs(ta - tb), axis=2) / den
    w = np.unravel_index(int(np.argmax(e)), e.shape)
    return float(e.max()), (int(w[0]), int(items[w[1]]))


def accuracy_items(p, n):
    """Work-order indices of n triplets spread over every hierarchy size and m_max:
    for each m_max, the cheapest triplet of the smallest, a middle and the largest
    l_max class, then triplets evenly spread over the cost-sorted order (without
    its most expensive tenth, whose rtol-1e-8 runs take minutes on a CPU core)."""
    order, kk = cost_order(p)
    cls = pair_order_classes(p)
    pick = []
    if cls is not None:
        ms = sorted({c[1] for c in cls})
        for m in ms:
            ls = sorted({c[0] for c in cls if c[1] == m})
            for L in (ls[0], ls[len(ls) // 2], ls[-1]):
                cand = [t for t in range(len(cls)) if cls[t] == (L, m)]
                pick.append(min(cand, key=lambda t: kk[t]))
    rest = max(0, n - len(pick))
    lo = len(order) // 10
    if rest:
        for q in np.linspace(lo, len(order) - 1, rest).astype(int):
            pick.append(int(order[q]))
    out = []
    for t in pick:
        if int(t) not in out:
            out.append(int(t))
    return np.array(out, dtype=np.int64)


# ---------------------------------------------------------------- oracle side (CPU)

def oracle_problem(cfg, overrides, fo=None, threads=None):
    """The workload built with the oracle library alone (its input provider is the
    same C source as the product's), first-order tables from the oracle or given."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from song_gb300 import capi
    from song_gb300.problem import config_problem
    oracle.build()
    oracle.load()
    host = capi.bind(C.CDLL(oracle.LIB), host_only=True)
    p = config_problem(cfg, lib=host, **overrides)
    if fo is None:
        fo = oracle.first_order(p, nthreads=threads or os.cpu_count())
    p.set_first_order(fo)
    return p


def accuracy_worker(cfg, overrides, fo_path, items_path, out_path, threads):
    """Spawned process: the oracle at rtol 1e-8 on the sample triplets."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    p = oracle_problem(cfg, overrides, fo=np.load(fo_path))
    items = np.load(items_path)
    t0 = time.perf_counter()
    ref, st = oracle.evolve(p, nthreads=threads, items=items, rtol=1e-8)
    np.savez(out_path, ref=ref, status=st["status"], seconds=time.perf_counter() - t0)


def stratified(order, m, offset):
    """m triplets, every (n/m)-th of the cost-sorted order starting at offset (mod the
    stride), most expensive first: the sample carries the workload's cost
    distribution, and the dynamic schedule starts its longest triplets first."""
    n = len(order)
    stride = max(1, n // max(1, m))
    return order[(offset % stride)::stride][:m], stride


def cpu_sample(p, m, threads, offset=0):
    """The oracle on a cost-stratified sample of m triplets of the workload.
    Returns (triplets/s, items, seconds, stride)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    order, _ = cost_order(p)
    pick, stride = stratified(order, m, offset)
    t0 = time.perf_counter()
    oracle.evolve(p, nthreads=threads, items=pick)
    dt = time.perf_counter() - t0
    return len(pick) / dt, len(pick), dt, stride


# ---------------------------------------------------------------- GPU side

def ctx_create(lib, p, precision, launch=None):
    from song_gb300 import capi
    c = C.c_void_p()
    err = capi.errbuf()
    if lib.song2_ctx_create_ex(C.byref(p.spec), C.byref(p.tables), precision,
                               C.byref(launch) if launch is not None else None, 0, 1, C.byref(c), err):
        raise RuntimeError(err.value.decode())
    return c


def autotune(lib, p, precision, sample):
    """song2_autotune's pick for this workload (untimed set-up)."""
    from song_gb300 import capi
    best = capi.Launch()
    ms = C.c_double()
    err = capi.errbuf()
    if lib.song2_autotune(C.byref(p.spec), C.byref(p.tables), precision, sample, C.byref(best), C.byref(ms), err):
        raise RuntimeError(err.value.decode())
    return best, ms.value


def run_parts(lib, c, parts, n_parts, torch, flush):
    """Run the given parts one per step, L2 flushed before each; device ms per part
    and launches in the timed region."""
    from song_gb300 import capi
    err = capi.errbuf()
    ms, launches = [], 0
    torch.cuda.synchronize()
    for q in parts:
        if flush is not None:
            flush.zero_()
            torch.cuda.synchronize()
        if lib.song2_ctx_run_part(c, int(q), n_parts, None, err):
            raise RuntimeError(err.value.decode())
        ms.append(lib.song2_ctx_last_kernel_ms(c))
        launches += lib.song2_ctx_last_launches(c)
    torch.cuda.synchronize()
    return ms, launches


def run_overlapped(lib, ctxs, parts, n_parts, torch):
    """The parts enqueued without waiting, part q on context q % len(ctxs) and on
    that context's stream, so that the last triplets of one part overlap the first
    ones of the next (the contexts have separate scratch); device time between one
    pair of CUDA events around all of them, and the evolver launches enqueued."""
    from song_gb300 import capi
    err = capi.errbuf()
    streams = [torch.cuda.Stream() for _ in ctxs]
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    cur = torch.cuda.current_stream()
    torch.cuda.synchronize()
    start.record(cur)
    for s in streams:
        s.wait_event(start)
    launches = 0
    for q in parts:
        k = q % len(ctxs)
        if lib.song2_ctx_enqueue_part(ctxs[k], int(q), n_parts, C.c_void_p(streams[k].cuda_stream), err):
            raise RuntimeError(err.value.decode())
        launches += lib.song2_ctx_last_launches(ctxs[k])
    for s in streams:
        e = torch.cuda.Event()
        e.record(s)
        cur.wait_event(e)
    stop.record(cur)
    torch.cuda.synchronize()
    return start.elapsed_time(stop), launches


class _RtolView:
    """The problem with another ODE rtol (a spec copy sharing the grids and tables)."""

    def __init__(self, p, rtol):
        from song_gb300 import capi
        self.spec = capi.Spec.from_buffer_copy(p.spec)
        self.spec.rtol = rtol
        self.tables = p.tables


def contract_leg(lib, p, launch, parts, n_parts, n_ctx, items, torch):
    """The mixed form at CONTRACT_RTOL: device time of the given parts (overlapped
    like the headline run) and the sources of the accuracy sample."""
    from song_gb300 import capi
    v = _RtolView(p, CONTRACT_RTOL)
    ctxs = [ctx_create(lib, v, capi.SONG2_PREC_MIXED, launch) for _ in range(n_ctx)]
    try:
        for q in range(n_ctx):  # regroup (untimed)
            run_parts(lib, ctxs[q], [parts[q % len(parts)]], n_parts, torch, None)
        ms, _ = run_overlapped(lib, ctxs, parts, n_parts, torch)
        _, st = download_all(lib, ctxs, p)
    finally:
        for c in ctxs:
            lib.song2_ctx_destroy(c)
    ran = int(np.count_nonzero(st["n_steps"]))
    src_acc = None
    if items is not None and len(items):
        c = C.c_void_p()
        err = capi.errbuf()
        it = np.ascontiguousarray(items, dtype=np.int64)
        if lib.song2_ctx_create_list(C.byref(v.spec), C.byref(v.tables), capi.SONG2_PREC_MIXED,
                                     it.ctypes.data_as(C.POINTER(C.c_int64)), len(it), C.byref(c), err):
            raise RuntimeError(err.value.decode())
        try:
            if lib.song2_ctx_run(c, None, err):
                raise RuntimeError(err.value.decode())
            src_acc, _ = download(lib, c, p)
        finally:
            lib.song2_ctx_destroy(c)
    return {"ms": ms, "triplets": ran, "status_ok": bool(np.all(st["status"] == 0)), "src": src_acc}


BI_R_SIZE = 75          # r samples of the bispectrum integral (r_size of the shipped precision files)
BI_Q_LINSTEP = 0.4      # q step of the first-order transfers in units of 2 pi / (tau0 - tau_rec)


def bispectra_inputs(p, los, ls, fields):
    """Synthetic first-order inputs of the bispectrum: an r grid of BI_R_SIZE points
    around the last-scattering distance, a q grid with the step of CLASS's transfer
    sampling (q_linstep 0.4) inside the sources' k range, the primordial spectrum
    2 pi^2 A_s (q/0.05)^(n_s-1) / q^3 of the benchmark cosmology, and Sachs-Wolfe-like
    first-order transfers T_l(q) = j_l(q (tau0 - tau_rec)) / 3 (E: a tenth of it)."""
    from scipy.special import spherical_jn
    tau0, trec = los.tau0, los.tau_rec
    r = np.linspace(tau0 - 2.5 * trec, tau0 + 0.5 * trec, BI_R_SIZE)
    step = BI_Q_LINSTEP * 2 * np.pi / (tau0 - trec)
    q = np.arange(p.k[0] * 1.0001, p.k[-1], step)
    pk = 2 * np.pi ** 2 * 2.1e-9 * (q / 0.05) ** (0.966 - 1) / q ** 3
    T1 = np.zeros((len(fields), len(ls), len(q)))
    for f, fld in enumerate(fields):
        for i, l in enumerate(ls):
            T1[f, i] = spherical_jn(int(l), q * (tau0 - trec)) / 3.0 * (1.0 if fld == 0 else 0.1)
    return r, q, pk, T1


def bispectra_spec(fields, r, q, pk, T1):
    from song_gb300 import capi
    bs = capi.BispectraSpec()
    bf = np.array(fields, dtype=np.int32)
    T1 = np.ascontiguousarray(T1)
    bs.bf_size, bs.bf = len(fields), capi.iptr(bf)
    bs.r_size, bs.r = len(r), capi.dptr(r)
    bs.q_size, bs.q = len(q), capi.dptr(q)
    bs.pk, bs.transfer1 = capi.dptr(pk), capi.dptr(T1)
    bs.k1_interpolation = bs.k2_interpolation = capi.INTERP_LINEAR
    bs._keep = (bf, r, q, pk, T1)
    return bs


def bispectra_leg(lib, p, los, ls, h_los, d_t2, t2_host, torch, reps, cpu_l):
    """The intrinsic bispectrum (T, E) of this run's second-order transfers, still in
    HBM after the line of sight: first-order tables once per handle, then the k3, k2,
    k1, r integrals and the geometry timed over `reps` runs.  The CPU restatement on
    the same inputs with the l list cut to its first cpu_l multipoles, and the GPU on
    that same cut, compared."""
    from song_gb300 import capi
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    fields = [0, 1]
    r, q, pk, T1 = bispectra_inputs(p, los, ls, fields)
    bs = bispectra_spec(fields, r, q, pk, T1)
    err = capi.errbuf()
    bh = C.c_void_p()
    t0 = time.perf_counter()
    if lib.song2_bispectra_create(h_los, C.byref(bs), C.byref(bh), err):
        raise RuntimeError(err.value.decode())
    torch.cuda.synchronize()
    create_s = time.perf_counter() - t0
    try:
        n_out = lib.song2_bispectra_size(bh)
        d_b = torch.zeros(n_out, dtype=torch.float64, device="cuda")
        ms = []
        for i in range(reps + 1):
            if lib.song2_bispectra_run(bh, C.c_void_p(d_t2.data_ptr()), C.c_void_p(d_b.data_ptr()), None, err):
                raise RuntimeError(err.value.decode())
            if i:
                ms.append(lib.song2_bispectra_last_ms(bh))
        b_full = d_b.cpu().numpy()
    finally:
        lib.song2_bispectra_destroy(bh)
    n_conf = n_out // 8
    # the cut: the first cpu_l multipoles, their transfer types, the same k units
    n_types = lib.song2_transfer_types(C.byref(p.spec), C.byref(los), None, None, None)
    ty = np.zeros(n_types, dtype=np.int32)
    tl = np.zeros(n_types, dtype=np.int32)
    lib.song2_transfer_types(C.byref(p.spec), C.byref(los), capi.iptr(ty), None, None)
    lib.song2_transfer_types(C.byref(p.spec), C.byref(los), None, capi.iptr(tl), None)
    keep = tl <= ls[cpu_l - 1]
    t2 = t2_host.reshape(n_types, -1)[keep].ravel()
    ls_cut = np.ascontiguousarray(ls[:cpu_l])
    los_cut = capi.LosSpec()
    C.memmove(C.byref(los_cut), C.byref(los), C.sizeof(capi.LosSpec))
    los_cut.l_size, los_cut.l = cpu_l, capi.iptr(ls_cut)
    bs_cut = bispectra_spec(fields, r, q, pk, T1[:, :cpu_l])
    n_cut = lib.song2_bispectra_configs(cpu_l, capi.iptr(ls_cut), None, None, None) * 8
    g_cut = np.zeros(n_cut)
    t0 = time.perf_counter()
    if lib.song2_gpu_bispectra(C.byref(p.spec), C.byref(los_cut), C.byref(bs_cut), capi.dptr(t2),
                               capi.dptr(g_cut), err):
        raise RuntimeError(err.value.decode())
    gpu_cut_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    ref = oracle.bispectra(p, los_cut, bs_cut, t2, n_cut)
    cpu_s = time.perf_counter() - t0
    g, w = g_cut.reshape(8, -1), ref.reshape(8, -1)
    scale = np.max(np.abs(w), axis=1)
    rel = float(np.max(np.max(np.abs(g - w), axis=1) / np.where(scale > 0, scale, 1.0)))
    t_run = sum(ms) / len(ms) / 1e3
    return {
        "metric": "intrinsic bispectrum b_l1l2l3 of every (l1 >= l2 >= l3) configuration and field combination "
                  "per second (bispectra2)",
        "value": n_out / t_run, "unit": "bispectrum values/s", "ms_per_run": 1e3 * t_run, "runs": reps,
        "workload": {"second_order": "this run's transfer functions (line of sight above), T and E, in HBM",
                     "configurations": int(n_conf), "fields": "TT, TE, ... (2^3 combinations)",
                     "m_list": [int(x) for x in p.spec.m[:p.spec.m_size]],
                     "r_size": BI_R_SIZE, "q_size": int(len(q)),
                     "first_order": "synthetic Sachs-Wolfe-like T_l(q) = j_l(q (tau0 - tau_rec))/3, E a tenth",
                     "interpolation": "linear in k1, k2 and the Bessel functions (the shipped precision files)"},
        "create_s": create_s,
        "cpu_baseline": {"value": n_cut / cpu_s, "unit": "bispectrum values/s", "cores": os.cpu_count(),
                         "kind": "port",
                         "sample": f"the same inputs with the l list cut to its first {cpu_l} multipoles "
                                   f"({n_cut // 8} configurations): CPU {cpu_s:.2f} s, GPU one-shot "
                                   f"{gpu_cut_s:.2f} s including its Bessel tables"},
        "max_rel_err_vs_cpu": rel, "tolerance": 1e-8, "within_tolerance": bool(rel <= 1e-8),
    }


def los_leg(lib, p, src_host, torch, reps, cpu_share, bispectra=True, bi_cpu_l=3):
    """transfer2 on the device: projection tables built once, then the line-of-sight
    integral of the config's sources (already in HBM) timed over `reps` runs; the CPU
    restatement on a contiguous run of the heaviest pairs as the baseline, and the
    GPU transfers of those pairs checked against it."""
    from song_gb300 import capi
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    los = capi.LosSpec()
    lib.song2_los_defaults(C.byref(los), C.byref(p.spec), C.byref(p.tables))
    n_l = lib.song2_l_list(*LOS_L, None)
    ls = np.zeros(n_l, dtype=np.int32)
    lib.song2_l_list(*LOS_L, capi.iptr(ls))
    los.l_size = n_l
    los.l = capi.iptr(ls)
    err = capi.errbuf()
    n_pairs = len(p.k) * (len(p.k) + 1) // 2
    ksz = np.zeros(n_pairs, dtype=np.int32)
    n_units = lib.song2_transfer_k_grids(C.byref(p.spec), C.byref(los), capi.iptr(ksz), None, None, None, err)
    n_tt = lib.song2_transfer_types(C.byref(p.spec), C.byref(los), None, None, None)
    h = C.c_void_p()
    t0 = time.perf_counter()
    if lib.song2_los_create(C.byref(p.spec), C.byref(los), C.byref(h), err):
        raise RuntimeError(err.value.decode())
    create_s = time.perf_counter() - t0
    try:
        xs, nl1, nr = C.c_int(), C.c_int(), C.c_int()
        lib.song2_los_table_sizes(h, C.byref(xs), C.byref(nl1), None, None, C.byref(nr))
        n_out = lib.song2_los_transfer_size(h)
        d_src = torch.from_numpy(src_host).cuda()
        d_out = torch.zeros(n_out, dtype=torch.float64, device="cuda")
        ms = []
        for r in range(reps + 1):
            if lib.song2_los_run(h, C.c_void_p(d_src.data_ptr()), C.c_void_p(d_out.data_ptr()), None, err):
                raise RuntimeError(err.value.decode())
            if r:
                ms.append(lib.song2_los_last_ms(h))
        tables_ms = lib.song2_los_tables_ms(h)
        out = d_out.cpu().numpy()
        bi_line = None
        if bispectra:
            try:
                bi_line = bispectra_leg(lib, p, los, ls, h, d_out, out, torch, reps, bi_cpu_l)
            except Exception as ex:  # noqa: BLE001
                bi_line = {"error": str(ex)[:300]}
    finally:
        lib.song2_los_destroy(h)
        d_src = d_out = None
    t_run = sum(ms) / len(ms) / 1e3
    # CPU restatement on the heaviest pairs (the last ones), about cpu_share of the units
    cum = np.cumsum(ksz[::-1])
    n_last = int(np.searchsorted(cum, cpu_share * n_units)) + 1
    lo = n_pairs - n_last
    units_cpu = int(ksz[lo:].sum())
    t0 = time.perf_counter()
    ref = oracle.transfer(p, los, src_host, n_out, nthreads=os.cpu_count(), pairs=(lo, n_pairs))
    cpu_s = time.perf_counter() - t0
    u0 = int(ksz[:lo].sum())
    g = out.reshape(n_tt, n_units)[:, u0:]
    r_ = ref.reshape(n_tt, n_units)[:, u0:]
    scale = np.max(np.abs(r_), axis=1)
    ok = scale > 0
    rel = float(np.max(np.max(np.abs(g - r_), axis=1)[ok] / scale[ok])) if ok.any() else 0.0
    zero_bad = float(np.max(np.abs(g[~ok]))) if (~ok).any() else 0.0
    return {
        "metric": "second-order transfer functions T_lm(k1,k2,k) per second (transfer2 line of sight)",
        "value": n_out / t_run, "unit": "transfers/s", "ms_per_run": 1e3 * t_run, "runs": reps,
        "units_per_s": n_units / t_run,
        "workload": {"sources": "this run's mixed-form sources of every triplet (already in HBM)",
                     "pairs": n_pairs, "k_units": int(n_units), "transfer_types": int(n_tt),
                     "l_list": f"l_max {LOS_L[0]}, l_logstep {LOS_L[1]}, l_linstep {LOS_L[2]} ({n_l} l)",
                     "x_grid": f"{xs.value} nodes of 0.2 to x_max {los.x_max:.0f}",
                     "projection_rows": int(nr.value), "bessel_l1": int(nl1.value),
                     "sampling": "k3 class (q_linstep 0.45), tau = source sampling, linear interpolation "
                                 "(transfer2 defaults)"},
        "tables_ms": float(tables_ms), "create_s": create_s,
        "cpu_baseline": {"value": n_tt * units_cpu / (cpu_s), "unit": "transfers/s", "cores": os.cpu_count(),
                         "kind": "port", "sample": f"the {n_last} pairs of largest k1 ({units_cpu} of {n_units} "
                                                   f"k units; {cpu_s:.1f} s including the tables)"},
        "max_rel_err_vs_cpu": rel, "zero_rows_nonzero": zero_bad, "tolerance": 1e-9,
        "within_tolerance": bool(rel <= 1e-9 and zero_bad == 0.0),
        "bispectra": bi_line,
    }


def download_all(lib, ctxs, p):
    """Sources and stats of contexts that evolved disjoint triplets, combined."""
    src, st = None, None
    for c in ctxs:
        s1, t1 = download(lib, c, p)
        if src is None:
            src, st = s1, t1
        else:
            src += s1
            st = np.where(t1["n_steps"] > 0, t1, st)
    return src, st


def download(lib, c, p):
    from song_gb300 import capi
    err = capi.errbuf()
    stats = (capi.TripletStats * p.n_triplets)()
    src = np.zeros(p.tp2_size * p.per_type)
    if lib.song2_ctx_download(c, capi.dptr(src), stats, err):
        raise RuntimeError(err.value.decode())
    return src, np.frombuffer(stats, dtype=capi.STATS_DTYPE).copy()


def run_e2e(lib, p, precision):
    """song2_gpu_evolve with host tables and host nested slabs: wall time on the host
    around the synchronous call (it returns after its D2H copies and the scatter)."""
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
    t0 = time.perf_counter()
    if lib.song2_gpu_evolve(C.byref(p.spec), C.byref(p.tables), precision, C.cast(tp_level, C.c_void_p), st, err):
        raise RuntimeError(err.value.decode())
    return time.perf_counter() - t0, table_bytes(p), d2h


# ---------------------------------------------------------------- arms

def reference_arm(args, cfg_num, overrides, config):
    """The CPU restatement with all host threads: each step a cost-stratified sample
    of the workload (ms_per_step = the steps' measured wall time)."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    threads = os.cpu_count()
    p = oracle_problem(cfg_num, overrides, threads=threads)
    config["triplets_per_gpu"] = p.n_triplets
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    order, _ = cost_order(p)
    n = len(order)
    m = min(n, args.ref_step_items)
    stride = max(1, n // m)
    # warm-up steps: one cheap triplet each (untimed)
    for w in range(args.warmup):
        oracle.evolve(p, nthreads=threads, items=order[-1 - w:][:1])
    walls, counts = [], []
    for j in range(args.steps):
        # a different stratified sample per step: the offsets walk through the strata
        items, _ = stratified(order, m, (j * stride) // max(1, args.steps) + j)
        t0 = time.perf_counter()
        oracle.evolve(p, nthreads=threads, items=items)
        walls.append(time.perf_counter() - t0)
        counts.append(len(items))
    v = sum(counts) / sum(walls)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "triplets/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(walls) / len(walls),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (own background/recombination and first-order provider)", "config": config,
            "cpu_baseline": {"value": v, "unit": "triplets/s", "cores": threads, "kind": "port",
                             "sample": f"each step every {stride}-th triplet of the cost-sorted "
                                       f"{n}-triplet workload ({m} triplets, {statistics.mean(walls):.1f} s), "
                                       f"most expensive first, offsets differ per step"},
            "e2e": {"value": v, "unit": "triplets/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "reference (coccoinomane/song) does not build: its CLASS submodule class.git is empty; "
                    "this arm times the CPU restatement of its algorithm (oracle/) with all host threads, "
                    "inputs built by the oracle library alone"}
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    rank, world, local = dist_env()
    from song_gb300.problem import CONFIGS
    cfg = dict(CONFIGS[args.config])
    overrides, cfg_name = workload_overrides(args, cfg)
    n_parts = args.parts or args.steps
    config = {"workload": cfg_name, "triplets_per_gpu": None, "k_min": cfg["k_min"], "k_max": cfg["k_max"],
              "k_size": cfg["k_size"], "k3_size": cfg["k3_size"], "l_max": cfg["l_max"], "m": list(cfg["m"]),
              "rtol": cfg["rtol"], "tau_size": cfg["tau_size"], "sources": cfg["sources"],
              "l2": "not flushed between steps: a step's working set (the quadratic-source tables of the "
                    "resident triplets, the first-order table) exceeds L2", "rsa": args.rsa}
    if cfg.get("uneven"):
        config["uneven"] = "l_max = min(40, 8 + ceil(k tau_rec/2)), m_max from {0,2,4} (seeded), 96 classes"

    if args.impl == "reference":
        return reference_arm(args, args.config, overrides, config)

    import torch
    import torch.distributed as dist
    if world > 1:
        dist.init_process_group("nccl", init_method="env://")
        torch.cuda.set_device(local)
    else:
        torch.cuda.set_device(0)
    from song_gb300 import build, capi
    from song_gb300.problem import config_problem
    if rank == 0:
        build.build()
    if world > 1:
        dist.barrier()
    lib = capi.load()
    p = config_problem(args.config, **overrides)
    p.first_order_gpu()          # first-order tables from the GPU first-order mode (untimed set-up)
    n_trip = p.n_triplets
    config["triplets_per_gpu"] = n_trip
    config["parts"] = (f"{n_parts} cost-balanced parts, one per step, on {max(1, min(args.contexts, n_parts))} "
                       f"contexts and streams so that consecutive parts overlap (song2_ctx_enqueue_part); "
                       f"value = triplets / device time of all")

    # the rtol-1e-8 oracle check runs in a spawned CPU process during the GPU arms
    acc = None
    if rank == 0 and world == 1 and args.accuracy_sample > 0:
        tmp = tempfile.mkdtemp(prefix="song2_bench_")
        items = accuracy_items(p, args.accuracy_sample)
        np.save(os.path.join(tmp, "fo.npy"), p.fo)
        np.save(os.path.join(tmp, "items.npy"), items)
        out = os.path.join(tmp, "ref.npz")
        proc = mp.get_context("spawn").Process(
            target=accuracy_worker,
            args=(args.config, overrides, os.path.join(tmp, "fo.npy"), os.path.join(tmp, "items.npy"), out,
                  max(1, os.cpu_count() - 2)))
        proc.start()
        acc = (proc, items, out, time.perf_counter())

    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    launch = None
    if args.autotune_sample > 0:
        launch, tune_ms = autotune(lib, p, capi.SONG2_PREC_MIXED, args.autotune_sample)
        config["launch"] = {"warp_team": launch.warp_team, "teams_per_cta": launch.teams_per_cta,
                            "threads_per_team": launch.threads_per_team, "factors_in_smem": launch.lu_in_smem,
                            "autotune": f"song2_autotune on {args.autotune_sample} triplets ({tune_ms:.0f} ms)"}
    # several contexts (separate scratch, separate streams): part q runs on context q % n_ctx
    n_ctx = max(1, min(args.contexts, n_parts))
    pp = min(args.plain_parts or max(1, args.steps // 4), max(1, n_parts - 2))
    ctxs = [ctx_create(lib, p, capi.SONG2_PREC_MIXED, launch) for _ in range(n_ctx)]
    try:
        # warm-up (untimed): every context regroups its work list and runs parts
        for w in range(max(args.warmup, n_ctx)):
            q = w % n_parts
            run_parts(lib, ctxs[q % n_ctx], [q], n_parts, torch, None)
        if world > 1:
            dist.barrier()
        flush.zero_()
        with Clocks(local) as clk:
            ms_total, launches = run_overlapped(lib, ctxs, [s % n_parts for s in range(args.steps)], n_parts, torch)
        if world > 1:
            dist.barrier()
        src_mixed, st_mixed = download_all(lib, ctxs, p)
        # the mixed form on the parts the plain form is timed on (the ratio's numerator)
        ms_mixed_same = None
        if not args.no_plain:
            ms_mixed_same, _ = run_overlapped(lib, ctxs, list(range(pp)), n_parts, torch)
    finally:
        for c in ctxs:
            lib.song2_ctx_destroy(c)
    clocks = clk.summary()
    t_mixed = ms_total / 1e3
    tt = torch.tensor([t_mixed], dtype=torch.float64, device="cuda")
    if world > 1:
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    t_mixed = float(tt.item())
    trip_timed = n_trip * args.steps / n_parts
    value = world * trip_timed / t_mixed

    plain = None
    if not args.no_plain:
        cp = [ctx_create(lib, p, capi.SONG2_PREC_FP64) for _ in range(n_ctx)]
        # untimed warm-up on the last parts (not among the timed ones when there are enough)
        warm = [q for q in range(n_parts - n_ctx, n_parts) if q >= pp]
        try:
            for q in warm:
                run_parts(lib, cp[q % n_ctx], [q], n_parts, torch, None)
            _, st_warm = download_all(lib, cp, p)
            ms_plain, _ = run_overlapped(lib, cp, list(range(pp)), n_parts, torch)
            src_plain, st_plain = download_all(lib, cp, p)
        finally:
            for c in cp:
                lib.song2_ctx_destroy(c)
        # the triplets of the timed parts (without the untimed warm-up parts)
        ran = np.nonzero((st_plain["n_steps"] > 0) & (st_warm["n_steps"] == 0))[0]
        plain = {"parts": pp, "ms": [ms_plain], "ms_mixed_same_parts": ms_mixed_same, "src": src_plain,
                 "st": st_plain, "ran": ran}

    contract = None
    if args.contract_parts > 0:
        # its own partition into CONTRACT_PARTS parts, whatever --steps is
        cp_parts = list(range(min(args.contract_parts, CONTRACT_PARTS)))
        contract = contract_leg(lib, p, launch, cp_parts, CONTRACT_PARTS, len(cp_parts),
                                acc[1] if acc is not None else None, torch)
        contract["parts"] = f"{len(cp_parts)} of {CONTRACT_PARTS}"

    e2e = None
    if not args.no_e2e:
        te, h2d, d2h = run_e2e(lib, p, capi.SONG2_PREC_MIXED)
        tt = torch.tensor([te], dtype=torch.float64, device="cuda")
        if world > 1:
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        e2e = {"value": world * n_trip / float(tt.item()), "unit": "triplets/s",
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "note": "whole workload through song2_gpu_evolve (one call: set-up, upload, evolve, download, "
                       "scatter into the nested host slabs)"}

    los_line = None
    if rank == 0 and world == 1 and not args.no_los:
        try:
            los_line = los_leg(lib, p, src_mixed, torch, args.los_reps, args.los_cpu_share,
                               bispectra=not args.no_bispectra, bi_cpu_l=args.bi_cpu_l)
        except Exception as ex:  # noqa: BLE001
            los_line = {"error": str(ex)[:300]}

    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return 0

    peaks = measured_peaks()
    ms_step = 1e3 * t_mixed / args.steps
    # roofline of the dominant kernel: algorithmic bytes of one step (a part) over its time
    alg = algorithmic_bytes(p) * (trip_timed / n_trip) / args.steps
    hbm_peak = peaks.get("hbm_gbs")
    achieved = alg / (ms_step / 1e3) / 1e9
    # DRAM traffic of one step: the measured bytes per triplet of the reduced case, times
    # the triplets of a step (the traffic grows with the triplets: each writes and
    # re-reads its own quadratic-source table, which the resident CTAs' tables spill
    # from L2)
    traffic = DRAM_BYTES_PER_TRIPLET * trip_timed / args.steps
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak or 6800.0, "unit": "GB/s",
                "frac": achieved / (hbm_peak or 6800.0), "traffic": traffic,
                "traffic_note": "bytes per step: ncu dram__bytes_read+write per triplet of the reduced config-4 "
                                "case (10.8 MB) times the triplets of a step; the excess over the algorithmic "
                                "bytes is the per-triplet quadratic-source tables, written and re-read by their "
                                "CTA, spilling from L2; DRAM runs at 0.03 % of peak",
                "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if hbm_peak else "fallback 6800",
                "note": "the evolver is bound by the latency of its FP64 chains and the FP64 pipe, not by HBM; "
                        "bytes = first-order rows of every (k1,k2) pair + background + source writes"}
    steps_tot = int(st_mixed["n_steps"].sum())
    sm_mhz = (clocks or {}).get("sm_mhz") or 2070.0
    nsm = torch.cuda.get_device_properties(0).multi_processor_count
    fp64_flops = steps_tot * FP64_FLOPS_PER_STEP / t_mixed * (args.steps / n_parts)
    fp64_peak = FP64_WARP_INSTR_PER_SM_CYCLE * 32 * 2 * sm_mhz * 1e6 * nsm
    fp64_slots = steps_tot * FP64_WARP_INSTR_PER_STEP / t_mixed * (args.steps / n_parts)
    slot_peak = FP64_WARP_INSTR_PER_SM_CYCLE * sm_mhz * 1e6 * nsm
    fp32_flops = steps_tot * FP32_FLOPS_PER_STEP / t_mixed * (args.steps / n_parts)
    roofline_fp64 = {"bound": "fp64", "achieved": fp64_flops / 1e12, "peak": fp64_peak / 1e12, "unit": "TFLOP/s",
                     "frac": fp64_flops / fp64_peak, "issue_slots_frac": fp64_slots / slot_peak,
                     "fp32_tflops": fp32_flops / 1e12,
                     "note": "FP64 flops (FMA = 2) per NDF step from the ncu counters of this kernel; peak from "
                             "the DFMA probe (one FP64 warp instruction per ~19 SM cycles, any lane count); "
                             "issue_slots_frac counts FP64 warp instructions against that rate"}
    line = {"metric": METRIC, "value": value, "unit": "triplets/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64 (FP32 iteration-matrix factors)",
            "data": "synthetic (own background/recombination and first-order provider)", "config": config,
            "gpu_launches": int(launches), "clocks": clocks, "roofline": roofline, "roofline_fp64": roofline_fp64,
            "e2e": e2e,
            "status_ok": bool(np.all(st_mixed["status"] == 0)),
            "triplets_ok": bool(np.all(st_mixed["status"] == 0)),
            "counters": {"ndf_steps": steps_tot, "rhs": int(st_mixed["n_rhs"].sum()),
                         "jacobians": int(st_mixed["n_jac"].sum()), "factorisations": int(st_mixed["n_lu"].sum()),
                         "rejected": int(st_mixed["n_rejected"].sum())}}
    if plain is not None:
        t_plain = sum(plain["ms"]) / 1e3
        n_pl = len(plain["ran"])
        line["plain_fp64"] = {"value": world * n_pl / t_plain, "unit": "triplets/s",
                              "ms_per_step": 1e3 * t_plain / plain["parts"],
                              "parts": f"{plain['parts']} of {n_parts} ({n_pl} triplets)",
                              "status_ok": bool(np.all(plain["st"]["status"][plain["ran"]] == 0))}
        if plain["ms_mixed_same_parts"]:
            line["mixed_over_plain"] = t_plain / (plain["ms_mixed_same_parts"] / 1e3)
        if n_pl:
            e, _ = source_error(p, src_mixed, plain["src"], plain["ran"], floor=1e-10)
            line["mixed_vs_plain_max_rel"] = e
    if contract is not None:
        line["contract"] = {"rtol": CONTRACT_RTOL, "value": world * contract["triplets"] / (contract["ms"] / 1e3),
                            "unit": "triplets/s", "parts": contract["parts"], "triplets": contract["triplets"],
                            "ms": contract["ms"], "status_ok": contract["status_ok"], "bound": ERR_BOUND,
                            "note": "the mixed form at the rtol where every sampled source meets the bound "
                                    "(same launch and overlap as the headline run)"}
    if los_line is not None:
        line["transfer2"] = los_line
    if rank == 0 and world == 1:
        # the CPU leg: the oracle timed on a bounded sample (after the accuracy worker)
        if acc is not None:
            proc, items, out, t_start = acc
            proc.join()
            try:
                r = np.load(out)
                ref, stat = r["ref"], r["status"]
                worst = {}
                errs = {}
                e, w = source_error(p, src_mixed, ref, items)
                errs["mixed"], worst["mixed"] = e, w
                if plain is not None:
                    both = np.intersect1d(items, plain["ran"])
                    if len(both):
                        e, w = source_error(p, plain["src"], ref, both)
                        errs["plain_fp64"], worst["plain_fp64"] = e, w
                work = p.work_order()
                tp = p.tp_list()
                line["err_vs_fp64_oracle"] = dict(
                    errs, sample_triplets=len(items), oracle_rtol=1e-8, bound=ERR_BOUND,
                    within_bound=bool(errs["mixed"] <= ERR_BOUND and errs.get("plain_fp64", 0.0) <= ERR_BOUND),
                    worst={k: {"source": list(tp[v[0]]), "triplet": list(work[v[1]])} for k, v in worst.items()},
                    oracle_status_ok=bool(np.all(stat == 0)), oracle_seconds=float(r["seconds"]),
                    metric="max over source types and sampled triplets of max_tau|S - S_ref| / max_tau|S_ref|",
                    sample="for each m_max the cheapest triplet of the smallest, a middle and the largest l_max "
                           "class, then triplets spread over the cost-sorted order without its top tenth")
                if not line["err_vs_fp64_oracle"]["within_bound"]:
                    line["status_ok"] = False
                if contract is not None and contract["src"] is not None:
                    e, w = source_error(p, contract["src"], ref, items)
                    line["contract"]["err_vs_fp64_oracle"] = e
                    line["contract"]["worst"] = {"source": list(tp[w[0]]), "triplet": list(work[w[1]])}
                    line["contract"]["within_bound"] = bool(e <= ERR_BOUND)
            except (OSError, KeyError, ValueError) as ex:
                line["err_vs_fp64_oracle"] = {"error": str(ex)[:200]}
        try:
            v, n, dt, stride = cpu_sample(p, args.cpu_sample, os.cpu_count())
            line["cpu_baseline"] = {"value": v, "unit": "triplets/s", "cores": os.cpu_count(), "kind": "port",
                                    "sample": f"{n} triplets, every {stride}-th of the cost-sorted "
                                              f"{n_trip}-triplet workload, most expensive first ({dt:.1f} s)"}
        except Exception as ex:  # noqa: BLE001
            line["cpu_baseline"] = {"value": None, "error": str(ex)[:200]}
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
