"""Build recipe for the GB300 overlap engine and its command-line front end.

    python -m canu_gb300.build          # everything
    python -m canu_gb300.build --lib    # only liboic_gpu.so

Outputs (git-ignored) go to canu_gb300/_build/:
    liboic_gpu.so      the C-ABI library (include/oic_gpu.h), sm_103a kernels
    overlapInCore      the drop-in command line, linked against the library
    oic_synth          the synthetic read generator
    oic_kmers          frequent k-mers of a read container (the -k skip file)
    oic_merge          merges the outputs of independent jobs (.ovb blocks, .oc counts)
    oic_store_build    the overlap-store build's record pass: filter, swapped copies, sort

Each translation unit is compiled in parallel; nvcc targets exactly sm_103a.
"""
import argparse
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_build")
CSRC = os.path.join(HERE, "csrc")
INC = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-O3",
           "--expt-relaxed-constexpr", "-I" + INC, "-I" + CSRC]
CU_SOURCES = ["oic_prims.cu", "oic_hash.cu", "oic_seed.cu", "oic_pairs.cu", "oic_capi.cu", "oic_noalloc.cu",
              "oic_filter.cu", "oic_kmers.cu", "oic_store.cu"]
HOST_SOURCES = ["oic_ovfile.cpp"]   # canu_gb300/host: host-only parts of the library


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs += [os.path.join(INC, f) for f in os.listdir(INC) if f.endswith(".h")]
    return hs


def build_lib(verbose=False, extra=()):
    os.makedirs(OUT, exist_ok=True)
    nv = nvcc()
    hdrs = _headers()
    objs = []
    jobs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src.replace(".cu", ".o"))
        objs.append(o)
        if _stale(o, [s] + hdrs):
            jobs.append([nv] + ARCH + NVFLAGS + list(extra) + ["-c", s, "-o", o])
    for src in HOST_SOURCES:
        s = os.path.join(HERE, "host", src)
        o = os.path.join(OUT, src.replace(".cpp", ".o"))
        objs.append(o)
        if _stale(o, [s] + hdrs):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-I" + INC, "-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    lib = os.path.join(OUT, "liboic_gpu.so")
    if _stale(lib, objs):
        _run([nv] + ARCH + ["-shared", "-o", lib] + objs + ["-lcudart"])
    return lib


def build_synth():
    """The synthetic read generator (host only; no CUDA)."""
    os.makedirs(OUT, exist_ok=True)
    syn_src = os.path.join(HERE, "synth", "oic_synth.cpp")
    syn = os.path.join(OUT, "oic_synth")
    if _stale(syn, [syn_src, os.path.join(INC, "oic_seqdb.h")]):
        _run(["g++", "-O2", "-std=c++17", "-I" + INC, "-o", syn, syn_src])
    return syn


def build_importer():
    """The FASTA / FASTQ importer into the read container (host only; no CUDA)."""
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(HERE, "host", "oic_seqdb_import.cpp")
    exe = os.path.join(OUT, "oic_seqdb_import")
    if _stale(exe, [src, os.path.join(INC, "oic_seqdb.h")]):
        _run(["g++", "-O2", "-std=c++17", "-Wall", "-I" + INC, "-o", exe, src])
    return exe


def build_tools():
    """The command-line tools, linked against liboic_gpu.so: overlapInCore (the drop-in),
    oic_kmers (frequent k-mers), oic_merge (merges independent jobs' outputs) and
    oic_store_build (the overlap store); and, host only, the read generator and the
    FASTA / FASTQ importer (oic_seqdb_import)."""
    os.makedirs(OUT, exist_ok=True)
    nv = nvcc()
    cuda_home = os.path.dirname(os.path.dirname(os.path.realpath(nv)))
    lib = os.path.join(OUT, "liboic_gpu.so")
    tools = {"overlapInCore": "overlapInCore.cpp", "oic_kmers": "oic_kmers.cpp", "oic_merge": "oic_merge.cpp",
             "oic_store_build": "oic_store_build.cpp"}
    jobs = []
    for name, src in tools.items():
        s = os.path.join(HERE, "host", src)
        t = os.path.join(OUT, name)
        if _stale(t, [s, lib] + _headers()):
            jobs.append(["g++", "-O2", "-std=c++17", "-Wall", "-I" + INC, "-o", t, s, "-L" + OUT, "-loic_gpu",
                         "-Wl,-rpath,$ORIGIN", "-L" + os.path.join(cuda_home, "lib64"), "-lcudart"])
    with ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        list(ex.map(_run, jobs))
    syn = build_synth()
    build_importer()
    return os.path.join(OUT, "overlapInCore"), syn


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--lib", action="store_true")
    ap.add_argument("-v", action="store_true")
    a = ap.parse_args(argv)
    print(build_lib(verbose=a.v))
    if not a.lib:
        print(*build_tools())


if __name__ == "__main__":
    sys.exit(main())
