"""Build the in-tree shared library song_gb300/_build/libsong2.so.

Host C is compiled with gcc, the CUDA translation units with nvcc for sm_103a
only (one -gencode), in parallel; the result is linked with the static CUDA
runtime so the library carries no dependency on torch.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
INC = os.path.join(ROOT, "include")
LIB = os.path.join(OUT, "libsong2.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-v"]
CC_FLAGS = ["-O2", "-fPIC", "-std=c11", "-Wall"]

C_SOURCES = ["song2_host.c", "song2_transfer_host.c", "song2_params.c", "song2_output.c"]
CU_SOURCES = ["song2_k_block_f.cu", "song2_k_block_d.cu", "song2_k_class_f.cu", "song2_k_class_d.cu",
              "song2_k_class2_f.cu", "song2_k_class2_d.cu", "song2_k_block2_f.cu", "song2_k_block2_d.cu",
              "song2_k_warp_f.cu", "song2_k_warp_d.cu", "song2_k_team_f.cu", "song2_k_team_d.cu",
              "song2_launch.cu", "song2_capi.cu", "song2_los.cu", "song2_bispectra.cu"]


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _run(cmd, log):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    with open(log, "w") as f:
        f.write(" ".join(cmd) + "\n" + p.stdout)
    if p.returncode != 0:
        sys.stderr.write(p.stdout)
        raise RuntimeError(f"build step failed: {' '.join(cmd)}")
    return p.stdout


# Diagnostic variant: the same library with the evolver's per-phase cycle
# counters compiled in (song2_ctx_phase_cycles), built into its own directory.
PHASE_OUT = os.path.join(HERE, "_build_phase")


def sources_newer_than_lib(lib=LIB):
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INC, "song2.h")]
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, phase_timers=False):
    out = PHASE_OUT if phase_timers else OUT
    lib = os.path.join(out, "libsong2.so")
    if not force and not sources_newer_than_lib(lib):
        return lib
    os.makedirs(out, exist_ok=True)
    extra = ["-DSONG2_PHASE_TIMERS"] if phase_timers else []
    nvcc = _nvcc()
    jobs = []
    objs = []
    for f in C_SOURCES:
        o = os.path.join(out, f + ".o")
        objs.append(o)
        jobs.append((["gcc", *CC_FLAGS, "-I", INC, "-c", os.path.join(CSRC, f), "-o", o], o + ".log"))
    for f in CU_SOURCES:
        o = os.path.join(out, f + ".o")
        objs.append(o)
        jobs.append(([nvcc, *ARCH, *NVCC_FLAGS, *extra, "-I", INC, "-I", CSRC, "-c", os.path.join(CSRC, f),
                      "-o", o], o + ".log"))
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        outs = list(ex.map(lambda j: _run(*j), jobs))
    if verbose:
        for o in outs:
            print(o)
    tmp = lib + ".tmp"
    _run([nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lm"], os.path.join(out, "link.log"))
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv, phase_timers="--phase-timers" in sys.argv))
