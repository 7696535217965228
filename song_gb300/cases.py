"""Fixed benchmark cases of the library, small enough to profile kernel by kernel.

    python -m song_gb300.cases evolver [--k-size 6] [--precision mixed|fp64] [--runs 2]
        config-4 hierarchy classes (l_max up to 40, m_max from {0,2,4}) on a
        reduced k grid: one context, whole runs of the persistent evolver.
    python -m song_gb300.cases los [--k-size 16] [--runs 3]
        the line-of-sight integral (transfer2) of config-4 geometry on a reduced k
        grid with seeded sources: projection tables once, then whole runs.
    python -m song_gb300.cases bispectra [--k-size 50] [--l-max 2000] [--runs 2]
        the intrinsic bispectrum (T, E; m <= 4) of seeded second-order transfers
        on config-4 geometry: line-of-sight tables and first-order tables once,
        then whole runs of the k3, k2, k1/r integrals and the symmetrisation.
    python -m song_gb300.cases phases [--config 4] [--parts 20]
        the per-phase clock64 cycle table of the evolver (a separate build with
        the phase timers compiled in), over one part of the workload.

Each prints the device time of every run and the work it did.
"""
import argparse
import ctypes as C
import os
import sys

import numpy as np

PHASES = ["SETUP", "QTAB", "IC", "START", "RESCALE", "FACT", "PRED", "PREP", "WS", "ROWS", "SOLVE", "NUPD", "JAC",
          "ERR", "ACCEPT", "OUT_RHS", "OUT_QS", "OUT_STORE", "CTRL", "ITEM", "SOLVE_BACK", "SOLVE_CORE",
          "FACT_CHAIN"]


def evolver(args):
    from song_gb300 import capi
    from song_gb300.problem import config_problem
    lib = capi.load()
    p = config_problem(4, k_size=args.k_size)
    p.first_order_gpu()
    prec = capi.SONG2_PREC_MIXED if args.precision == "mixed" else capi.SONG2_PREC_FP64
    c = C.c_void_p()
    err = capi.errbuf()
    launch = capi.Launch(0, 1, 256, 1)
    if lib.song2_ctx_create_ex(C.byref(p.spec), C.byref(p.tables), prec, C.byref(launch), 0, 1, C.byref(c), err):
        raise RuntimeError(err.value.decode())
    try:
        for r in range(args.runs):
            if lib.song2_ctx_run(c, None, err):
                raise RuntimeError(err.value.decode())
            print(f"run {r}: {lib.song2_ctx_last_kernel_ms(c):.1f} ms, {lib.song2_ctx_last_launches(c)} launches",
                  flush=True)
        st = (capi.TripletStats * p.n_triplets)()
        src = np.zeros(p.tp2_size * p.per_type)
        lib.song2_ctx_download(c, capi.dptr(src), st, err)
    finally:
        lib.song2_ctx_destroy(c)
    st = np.frombuffer(st, dtype=capi.STATS_DTYPE)
    print(f"triplets {p.n_triplets}, NDF steps {int(st['n_steps'].sum())}, statuses {np.unique(st['status'])}")


def los(args):
    import torch
    from song_gb300 import capi
    from song_gb300.problem import config_problem
    lib = capi.load()
    p = config_problem(4, k_size=args.k_size)
    los = capi.LosSpec()
    lib.song2_los_defaults(C.byref(los), C.byref(p.spec), C.byref(p.tables))
    n = lib.song2_l_list(2000, 1.25, 36, None)
    ls = np.zeros(n, dtype=np.int32)
    lib.song2_l_list(2000, 1.25, 36, capi.iptr(ls))
    los.l_size = n
    los.l = capi.iptr(ls)
    err = capi.errbuf()
    h = C.c_void_p()
    if lib.song2_los_create(C.byref(p.spec), C.byref(los), C.byref(h), err):
        raise RuntimeError(err.value.decode())
    try:
        rng = np.random.default_rng(3)
        src = torch.from_numpy(rng.normal(size=p.tp2_size * p.per_type)).cuda()
        out = torch.zeros(lib.song2_los_transfer_size(h), dtype=torch.float64, device="cuda")
        for r in range(args.runs):
            if lib.song2_los_run(h, C.c_void_p(src.data_ptr()), C.c_void_p(out.data_ptr()), None, err):
                raise RuntimeError(err.value.decode())
            print(f"run {r}: {lib.song2_los_last_ms(h):.2f} ms", flush=True)
        print(f"tables {lib.song2_los_tables_ms(h):.2f} ms, transfers {out.numel()}")
    finally:
        lib.song2_los_destroy(h)


def bispectra(args):
    import torch
    from song_gb300 import capi
    from song_gb300.problem import config_problem
    from scipy.special import spherical_jn
    lib = capi.load()
    p = config_problem(4, k_size=args.k_size)
    los = capi.LosSpec()
    lib.song2_los_defaults(C.byref(los), C.byref(p.spec), C.byref(p.tables))
    n = lib.song2_l_list(args.l_max, 1.25, 36, None)
    ls = np.zeros(n, dtype=np.int32)
    lib.song2_l_list(args.l_max, 1.25, 36, capi.iptr(ls))
    los.l_size = n
    los.l = capi.iptr(ls)
    err = capi.errbuf()
    h = C.c_void_p()
    if lib.song2_los_create(C.byref(p.spec), C.byref(los), C.byref(h), err):
        raise RuntimeError(err.value.decode())
    b = C.c_void_p()
    try:
        tau0, trec = los.tau0, los.tau_rec
        r = np.linspace(tau0 - 2.5 * trec, tau0 + 0.5 * trec, 75)
        q = np.arange(p.k[0] * 1.0001, p.k[-1], 0.4 * 2 * np.pi / (tau0 - trec))
        pk = 2 * np.pi ** 2 * 2.1e-9 * (q / 0.05) ** (0.966 - 1) / q ** 3
        T1 = np.stack([np.stack([spherical_jn(int(l), q * (tau0 - trec)) / 3.0 * s_ for l in ls])
                       for s_ in (1.0, 0.1)])
        bf = np.array([0, 1], dtype=np.int32)
        bs = capi.BispectraSpec(2, capi.iptr(bf), len(r), capi.dptr(r), len(q), capi.dptr(q), capi.dptr(pk),
                                capi.dptr(np.ascontiguousarray(T1)), capi.INTERP_LINEAR, capi.INTERP_LINEAR)
        if lib.song2_bispectra_create(h, C.byref(bs), C.byref(b), err):
            raise RuntimeError(err.value.decode())
        rng = np.random.default_rng(3)
        t2 = torch.from_numpy(rng.normal(size=lib.song2_los_transfer_size(h))).cuda()
        out = torch.zeros(lib.song2_bispectra_size(b), dtype=torch.float64, device="cuda")
        for i in range(args.runs):
            if lib.song2_bispectra_run(b, C.c_void_p(t2.data_ptr()), C.c_void_p(out.data_ptr()), None, err):
                raise RuntimeError(err.value.decode())
            print(f"run {i}: {lib.song2_bispectra_last_ms(b):.1f} ms", flush=True)
        print(f"l {n}, r {len(r)}, q {len(q)}, k {len(p.k)}, bispectrum values {out.numel()}")
    finally:
        if b:
            lib.song2_bispectra_destroy(b)
        lib.song2_los_destroy(h)


def phases(args):
    from song_gb300 import build
    here = os.path.dirname(os.path.abspath(__file__))
    os.environ["SONG2_LIB"] = os.path.join(here, "_build_phase", "libsong2.so")
    build.build(phase_timers=True)
    from song_gb300 import capi
    from song_gb300.problem import config_problem
    lib = capi.load()
    p = config_problem(args.config)
    p.first_order_gpu()
    for prec, name in ((capi.SONG2_PREC_MIXED, "mixed"), (capi.SONG2_PREC_FP64, "plain FP64")):
        c = C.c_void_p()
        err = capi.errbuf()
        if lib.song2_ctx_create_shard(C.byref(p.spec), C.byref(p.tables), prec, 0, args.parts, C.byref(c), err):
            raise RuntimeError(err.value.decode())
        try:
            if lib.song2_ctx_run(c, None, err):
                raise RuntimeError(err.value.decode())
            ms = lib.song2_ctx_last_kernel_ms(c)
            stats = (capi.TripletStats * p.n_triplets)()
            src = np.zeros(p.tp2_size * p.per_type)
            lib.song2_ctx_download(c, capi.dptr(src), stats, err)
            ph = (C.c_uint64 * 64)()
            n = lib.song2_ctx_phase_cycles(c, ph, 64)
        finally:
            lib.song2_ctx_destroy(c)
        st = np.frombuffer(stats, dtype=capi.STATS_DTYPE)
        done = st[st["n_steps"] > 0]
        steps = int(done["n_steps"].sum())
        ph = np.array(ph[:2 * n], dtype=np.float64).reshape(n, 2)
        item = PHASES.index("ITEM")
        tot = ph[:item, 0].sum() + ph[item + 1:, 0].sum()
        print(f"{name}: {ms:.1f} ms, {len(done)} triplets (shard 0 of {args.parts}), NDF steps {steps}")
        print(f"  {'phase':10s} {'cycles/step':>12s} {'share':>7s} {'visits/step':>11s} {'cycles/visit':>12s}")
        for i, nm in enumerate(PHASES[:n]):
            if ph[i, 1] == 0 or i == item:
                continue
            print(f"  {nm:10s} {ph[i, 0] / steps:12.0f} {100 * ph[i, 0] / tot:6.1f}% {ph[i, 1] / steps:11.3f} "
                  f"{ph[i, 0] / ph[i, 1]:12.0f}")
        print(f"  marked cycles per NDF step {tot / steps:.0f} (a triplet's CTA, summed over its phases)", flush=True)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("case", choices=["evolver", "los", "bispectra", "phases"])
    ap.add_argument("--l-max", type=int, default=2000)
    ap.add_argument("--k-size", type=int, default=None)
    ap.add_argument("--precision", choices=["mixed", "fp64"], default="mixed")
    ap.add_argument("--runs", type=int, default=None)
    ap.add_argument("--config", type=int, default=4)
    ap.add_argument("--parts", type=int, default=20)
    args = ap.parse_args(argv)
    if args.case == "evolver":
        args.k_size = args.k_size or 6
        args.runs = args.runs or 2
        evolver(args)
    elif args.case == "los":
        args.k_size = args.k_size or 16
        args.runs = args.runs or 3
        los(args)
    elif args.case == "bispectra":
        args.k_size = args.k_size or 50
        args.runs = args.runs or 2
        bispectra(args)
    else:
        phases(args)
    return 0


if __name__ == "__main__":
    sys.exit(main())
