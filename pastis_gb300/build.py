"""Build recipe for the native parts of pastis_gb300 (in-tree, no cmake).

libpastis_gb300.so   CUDA kernels + C ABI (nvcc, sm_103a only)
libpastis_synth.so   synthetic data generator (gcc, OpenMP)
libpastis_host.so    C++ host side: PWAlign mirror and pw_aln_batch driver

All outputs go to pastis_gb300/_build/.  Compiles run in parallel.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INC = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INC]
CUDA_UNITS = ("pg_api.cu", "pg_stat.cu", "pg_dir.cu", "pg_dir_ga.cu", "pg_dir_sw.cu", "pg_filter.cu", "pg_kmer.cu", "pg_fasta.cu")


def _steps():
    """Build steps in dependency order; each step is a list of independent
    jobs (output name, command without -o, dependencies) run in parallel."""
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers += [os.path.join(INC, "pastis_gb300.h")]
    objs = []
    compile_jobs = []
    for u in CUDA_UNITS:
        src = os.path.join(CSRC, u)
        obj = u.replace(".cu", ".o")
        objs.append(os.path.join(BUILD, obj))
        compile_jobs.append((obj, [NVCC] + NVCC_FLAGS + ["-c", src], [src] + headers))
    synth = os.path.join(CSRC, "synth.c")
    compile_jobs.append(("libpastis_synth.so",
                         ["gcc", "-O3", "-std=c99", "-fopenmp", "-fPIC", "-shared", "-I", INC,
                          synth, "-lm"],
                         [synth, os.path.join(INC, "pastis_gb300_synth.h")]))
    link = [("libpastis_gb300.so", [NVCC] + ARCH + ["-shared"] + objs, objs)]
    host_src = [os.path.join(CSRC, "host.cpp")]
    host = [("libpastis_host.so",
             ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I", INC] + host_src
             + ["-L", BUILD, "-lpastis_gb300", "-Wl,-rpath,$ORIGIN"],
             host_src + [os.path.join(BUILD, "libpastis_gb300.so"),
                         os.path.join(INC, "pastis_gb300_pwalign.hpp"),
                         os.path.join(INC, "pastis_gb300_host.h"),
                         os.path.join(INC, "pastis_gb300.h")])]
    return [compile_jobs, link, host]


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force=False, verbose=False, only=None):
    """Build every library, or only the outputs named in ``only`` (e.g.
    {"libpastis_synth.so"}: the generator alone, no CUDA compile)."""
    os.makedirs(BUILD, exist_ok=True)
    for jobs in _steps():
        procs = []
        for name, cmd, deps in jobs:
            if only is not None and name not in only:
                continue
            out = os.path.join(BUILD, name)
            if not force and not _stale(out, deps):
                continue
            tmp = out + ".tmp%d" % os.getpid() + os.path.splitext(name)[1]
            full = cmd[:1] + ["-o", tmp] + cmd[1:]
            if verbose:
                print(" ".join(full), file=sys.stderr)
            procs.append((subprocess.Popen(full, stdout=subprocess.PIPE, stderr=subprocess.STDOUT),
                          tmp, out, name))
        for p, tmp, out, name in procs:
            log = p.communicate()[0].decode(errors="replace")
            if p.returncode != 0:
                raise RuntimeError("building %s failed:\n%s" % (name, log))
            os.replace(tmp, out)
    return BUILD


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print(BUILD)
