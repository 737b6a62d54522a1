"""Build the engine in-tree: cuspx_gb300/lib/libcuspx.so plus one NIST api.h
drop-in library per parameter set, lib/libspx_<set>.so.

sm_103a only (-gencode arch=compute_103a,code=sm_103a).  The twelve hash
family instantiations are separate objects compiled in parallel; objects are
rebuilt only when a source or header is newer.

    python -m cuspx_gb300.build [-v] [-j N]
"""
import concurrent.futures
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INC = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "lib")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-diag-suppress", "20050"] + ARCH
CXX_FLAGS = ["-std=c++17", "-O2", "-fPIC", "-Wall"]

SET_NAMES = [f"{h}-{s}-{m}" for h in ("sha256", "shake256") for s in ("128s", "128f", "192s", "192f", "256s", "256f")
             for m in ("simple", "robust")]


def _nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s" % (" ".join(cmd), r.stdout))
    if verbose and r.stdout.strip():
        print(r.stdout, flush=True)
    return r.stdout


def build(verbose=False, jobs=None, ptxas_verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIB, exist_ok=True)
    nvcc = _nvcc()
    headers = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(INC, "*.h"))
    extra = ["-Xptxas", "-v"] if ptxas_verbose else []
    # extra device flags (A/B experiments); a change of flags rebuilds everything
    user = os.environ.get("CUSPX_NVCC_FLAGS", "").split()
    extra += user
    stamp = os.path.join(BUILD, "flags.stamp")
    prev = open(stamp).read() if os.path.exists(stamp) else None
    if prev != " ".join(user):
        for o in glob.glob(os.path.join(BUILD, "*.o")):
            os.remove(o)
        with open(stamp, "w") as f:
            f.write(" ".join(user))
    steps = []
    fam_src = os.path.join(CSRC, "spx_family.cu")
    for h in (0, 1):
        for n in (16, 24, 32):
            for r in (0, 1):
                obj = os.path.join(BUILD, f"family_{h}_{n}_{r}.o")
                cmd = [nvcc] + NVCC_FLAGS + extra + [f"-DFAMILY_HASH={h}", f"-DFAMILY_N={n}", f"-DFAMILY_ROBUST={r}",
                                                     "-c", fam_src, "-o", obj]
                steps.append((obj, [fam_src] + headers, cmd))
    for src in ("engine.cu", "serve.cu", "calib.cu", "noalloc.cu"):
        s = os.path.join(CSRC, src)
        if os.path.exists(s):
            obj = os.path.join(BUILD, src.replace(".cu", ".o"))
            steps.append((obj, [s] + headers, [nvcc] + NVCC_FLAGS + extra + ["-c", s, "-o", obj]))
    for src in ("drbg.cpp",):
        s = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src.replace(".cpp", ".o"))
        steps.append((obj, [s] + headers, ["g++"] + CXX_FLAGS + ["-c", s, "-o", obj]))
    todo = [(o, c) for (o, d, c) in steps if _newer(o, d)]
    jobs = jobs or max(2, min(len(todo) or 1, os.cpu_count() or 4))
    with concurrent.futures.ThreadPoolExecutor(jobs) as ex:
        outs = list(ex.map(lambda oc: _run(oc[1], verbose), todo))
    if ptxas_verbose:
        for o in outs:
            print(o)
    objs = [o for (o, _, _) in steps]
    core = os.path.join(LIB, "libcuspx.so")
    if _newer(core, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", core] + objs + ["-lpthread"], verbose)
    api_src = os.path.join(CSRC, "api_dropin.cpp")
    drops = []
    for name in SET_NAMES:
        so = os.path.join(LIB, f"libspx_{name}.so")
        if _newer(so, [api_src, core] + headers):
            drops.append(["g++"] + CXX_FLAGS + ["-shared", f'-DCUSPX_SET_NAME="{name}"', api_src, "-o", so,
                                               "-L" + LIB, "-lcuspx", "-Wl,-rpath,$ORIGIN"])
    with concurrent.futures.ThreadPoolExecutor(jobs) as ex:
        list(ex.map(lambda c: _run(c, verbose), drops))
    return core


if __name__ == "__main__":
    v = "-v" in sys.argv
    j = None
    if "-j" in sys.argv:
        j = int(sys.argv[sys.argv.index("-j") + 1])
    print(build(verbose=v, jobs=j, ptxas_verbose="--ptxas" in sys.argv))
