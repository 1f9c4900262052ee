"""Build the native parts in-tree.

* ``locarna_gb300/_build/liblocarna_gb300.so``: the CUDA engine (sm_103a) and
  the C ABI of include/locarna_gb300.h;
* ``locarna_gb300/_build/liblcg_probe.so``: the int32 add+max rate probe the
  benchmark reports its integer roofline against (measurement only, not part
  of the engine);
* ``oracle/_build/liboracle.so``: the plain-C oracle (test infrastructure);
* ``oracle/_ref/*``: the reference's own sources compiled as an oracle, only
  where the reference sources are present (``oracle/build_ref.sh``).

Translation units are compiled in parallel; one ``-gencode`` for sm_103a.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "locarna_gb300")
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
ORACLE = os.path.join(ROOT, "oracle")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
GENCODE = "-gencode=arch=compute_103a,code=sm_103a"

# tuning defines for the CUDA sources, e.g. LCG_NVCC_DEFS="-DLCG_FILL_WARPS=4"
EXTRA_DEFS = os.environ.get("LCG_NVCC_DEFS", "").split()

CUDA_SOURCES = ["engine.cu", "sankoff_kernels.cu", "sankoff_sl_kernels.cu", "noalloc.cu",
                "pf_kernels.cu", "engine_pf.cu", "envelope.cu"]
PROBE_SOURCE = "microbench.cu"  # the measurement probe, a library of its own
HOST_SOURCES = ["host_prep.cpp"]  # C++ host-only translation units


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_engine(verbose=False, force=False, out=None, defs=None):
    """liblocarna_gb300.so in `out` (default the package's _build) with the
    extra defines `defs` (default $LCG_NVCC_DEFS)."""
    OUT = out or globals()["OUT"]
    EXTRA_DEFS = defs if defs is not None else globals()["EXTRA_DEFS"]
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h", ".hh"))]
    headers.append(os.path.join(ROOT, "include", "locarna_gb300.h"))
    objs = []
    jobs = []
    for src in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        if force or _newer(o, [s] + headers):
            jobs.append([NVCC, GENCODE, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-Xptxas", "-v" if verbose else "-O3"] + EXTRA_DEFS + ["-c", s, "-o", o])
    for src in HOST_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        if force or _newer(o, [s] + headers):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off",
                         "-I", os.path.join(ROOT, "include"), "-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        logs = list(ex.map(_run, jobs))
    if verbose:
        for log in logs:
            sys.stdout.write(log)
    lib = os.path.join(OUT, "liblocarna_gb300.so")
    if force or jobs or not os.path.exists(lib):
        _run([NVCC, GENCODE, "-shared", "-o", lib] + objs + ["-lcudart"])
    return lib


CLI_SOURCES = {"locarna": "locarna.cc", "locarna_p": "locarna_p.cc"}


def build_cli(force=False):
    """The locarna / locarna_p command lines (C++ over the C ABI), linked
    against liblocarna_gb300.so with an rpath to the build folder."""
    lib = build_engine()
    cli = os.path.join(PKG, "cli")
    hdrs = [os.path.join(cli, f) for f in os.listdir(cli) if f.endswith(".hh")]
    hdrs += [os.path.join(ROOT, "include", "locarna_gb300.h"), os.path.join(ROOT, "include", "locarna_gb300.hpp")]
    outs = []
    jobs = []
    for exe, src in CLI_SOURCES.items():
        s = os.path.join(cli, src)
        out = os.path.join(OUT, exe)
        outs.append(out)
        if force or _newer(out, [s, lib] + hdrs):
            jobs.append(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), s, "-o", out,
                         "-L", OUT, "-llocarna_gb300", "-Wl,-rpath," + OUT])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(_run, jobs))
    return outs


def build_probe(force=False):
    """The int32 add+max rate probe (lcg_probe_int_peak) as its own library."""
    os.makedirs(OUT, exist_ok=True)
    s = os.path.join(CSRC, PROBE_SOURCE)
    lib = os.path.join(OUT, "liblcg_probe.so")
    if force or _newer(lib, [s]):
        _run([NVCC, GENCODE, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", s, "-o", lib,
              "-lcudart"])
    return lib


def build_oracle():
    out = os.path.join(ORACLE, "_build")
    os.makedirs(out, exist_ok=True)
    hdr = os.path.join(ROOT, "include", "locarna_gb300.h")
    # the Sankoff oracle: the C restatement plus the k-best driver (C++, for
    # std::priority_queue's order of equal scores)
    lib = os.path.join(out, "liboracle.so")
    srcs = [os.path.join(ORACLE, "sankoff_oracle.c"), os.path.join(ORACLE, "kbest_oracle.cc")]
    if _newer(lib, srcs + [hdr]):
        obj = os.path.join(out, "sankoff_oracle.o")
        _run(["gcc", "-O2", "-std=c11", "-fPIC", "-ffp-contract=off", "-c", srcs[0], "-o", obj])
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", srcs[1], obj, "-o", lib, "-lm"])
    lib = os.path.join(out, "libpforacle.so")
    s = os.path.join(ORACLE, "pf_oracle.c")
    if _newer(lib, [s, hdr]):
        _run(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", s, "-o", lib, "-lm"])
    # the CPU port of the locarna pipeline (host table preparation + the C
    # restatement), timed by bench.py's reference arm
    port = os.path.join(out, "port_locarna")
    psrc = [os.path.join(ORACLE, "port_locarna.cc"), os.path.join(ORACLE, "prep_link.cc"),
            os.path.join(CSRC, "host_prep.cpp")]
    deps = psrc + [hdr, os.path.join(CSRC, "envelope.hh"), os.path.join(CSRC, "ribosum85_60.inc"), srcs[0]]
    if _newer(port, deps):
        _run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "include")] + psrc +
             [os.path.join(out, "sankoff_oracle.o"), "-o", port, "-lpthread", "-lm"])
    return os.path.join(out, "liboracle.so")


def reference_tree():
    """The reference source tree: $LOCARNA_REF, else a checkout named
    ``reference`` beside the repository."""
    return os.environ.get("LOCARNA_REF") or os.path.join(os.path.dirname(ROOT), "reference")


def build_reference_oracle():
    """Compile the reference sources as an oracle when they are present."""
    ref = reference_tree()
    if not os.path.isdir(os.path.join(ref, "src", "LocARNA")):
        return None
    _run(["bash", os.path.join(ORACLE, "build_ref.sh")])
    return os.path.join(ORACLE, "_ref")


def build_all(verbose=False):
    with ThreadPoolExecutor(max_workers=4) as ex:
        f1 = ex.submit(build_engine, verbose)
        f2 = ex.submit(build_oracle)
        f3 = ex.submit(build_reference_oracle)
        f4 = ex.submit(build_probe)
        r = f1.result(), f2.result(), f3.result(), f4.result()
    return r + (build_cli(),)


if __name__ == "__main__":
    print(build_all(verbose="-v" in sys.argv))
