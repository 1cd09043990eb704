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


def _targets():
    cu = [os.path.join(CSRC, f) for f in ("pg_api.cu", "pg_filter.cu")]
    cu_deps = cu + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")]
    cu_deps += [os.path.join(INC, "pastis_gb300.h")]
    host_src = [os.path.join(CSRC, "host.cpp")]
    return [
        ("libpastis_gb300.so",
         [NVCC] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
                          "-I", INC] + cu,
         cu_deps),
        ("libpastis_synth.so",
         ["gcc", "-O3", "-std=c99", "-fopenmp", "-fPIC", "-shared", "-I", INC,
          os.path.join(CSRC, "synth.c"), "-lm"],
         [os.path.join(CSRC, "synth.c"), os.path.join(INC, "pastis_gb300_synth.h")]),
        ("libpastis_host.so",
         ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I", INC] + host_src
         + ["-L", BUILD, "-lpastis_gb300", "-Wl,-rpath,$ORIGIN"],
         host_src + [os.path.join(INC, "pastis_gb300_pwalign.hpp"),
                     os.path.join(INC, "pastis_gb300.h")]),
    ]


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    targets = [t for t in _targets() if os.path.exists(t[2][0])]
    # the host library links against the CUDA library: build that first
    first = [t for t in targets if t[0] != "libpastis_host.so"]
    later = [t for t in targets if t[0] == "libpastis_host.so"]
    for group in (first, later):
        procs = []
        for name, cmd, deps in group:
            out = os.path.join(BUILD, name)
            if not force and not _stale(out, deps):
                continue
            tmp = out + ".tmp%d" % os.getpid()
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
