"""In-tree build of the native parts (no CMake, no torch extension machinery).

  spinwalk_gb300/libspinwalk_gpu.so   nvcc, sm_103a only, -fmad=false (bit-exact float order)
  spinwalk_gb300/spinwalk             the `spinwalk sim -c cfg.ini` command-line host (C++)
  oracle/liboracle.so                 the test oracle (g++), built here for tests and bench
  oracle/libsynth.so                  the synthetic phantom generator alone (the CPU reference
                                      arm of the benchmark makes its inputs with it)
  oracle/_ref/libref_sim.so           the reference's own sim(), only where its source tree is
                                      given by the SPINWALK_REF_SRC environment variable

Translation units compile in parallel; a unit is rebuilt when any source or header changed.
"""
import hashlib
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INC = os.path.join(ROOT, "include")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libspinwalk_gpu.so")
REF_TREE = os.environ.get("SPINWALK_REF_SRC", "")   # the SpinWalk source tree, if any

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", *ARCH, "-lineinfo", "-fmad=false",
              "-Xcompiler", "-fPIC,-ffp-contract=off,-fopenmp", f"-I{INC}", f"-I{CSRC}"]
CUDA_INC = "/usr/local/cuda/include"
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fopenmp", f"-I{INC}",
             f"-I{CSRC}", f"-I{CUDA_INC}"]
CLI = os.path.join(PKG, "spinwalk")

CU_UNITS = ["sw_kernels.cu", "sw_api.cu", "sw_noalloc.cu", "sw_tracks.cu", "sw_engine.cu",
            "sw_phantom_gpu.cu", "sw_minstd.cu", "sw_order.cu", "sw_tune.cu", "sw_pool.cu"]
CXX_UNITS = ["sw_host.cpp", "sw_phantom.cpp", "sw_config.cpp", "sw_h5.cpp", "sw_driver.cpp",
             "sw_mtjump.cpp"]


def _nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _digest(files, extra):
    h = hashlib.sha256()
    for f in sorted(files):
        with open(f, "rb") as fh:
            h.update(fh.read())
    h.update(" ".join(extra).encode())
    return h.hexdigest()[:16]


def _headers():
    out = [os.path.join(INC, f) for f in os.listdir(INC) if f.endswith(".h")]
    out += [os.path.join(CSRC, f) for f in os.listdir(CSRC)
            if f.endswith((".h", ".cuh"))]
    return out


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr.strip():
        print(r.stderr, file=sys.stderr)
    return r


def build_lib(verbose=False, force=False):
    os.makedirs(OBJ, exist_ok=True)
    nvcc = _nvcc()
    hdrs = _headers()
    jobs = []
    objs = []
    for u in CU_UNITS + CXX_UNITS:
        src = os.path.join(CSRC, u)
        is_cu = u.endswith(".cu")
        flags = NVCC_FLAGS if is_cu else CXX_FLAGS
        dig = _digest([src] + hdrs, flags)
        obj = os.path.join(OBJ, f"{u}.{dig}.o")
        objs.append(obj)
        if force or not os.path.exists(obj):
            cmd = ([nvcc, *flags, "-c", src, "-o", obj] if is_cu
                   else ["g++", *flags, "-c", src, "-o", obj])
            jobs.append(cmd)
    if jobs:
        with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            list(ex.map(lambda c: _run(c, verbose), jobs))
    stamp = _digest(objs, ["link"])
    stamp_file = LIB + ".stamp"
    if force or jobs or not os.path.exists(LIB) or not os.path.exists(stamp_file) or \
            open(stamp_file).read() != stamp:
        tmp = LIB + ".tmp"
        _run([nvcc, "-shared", *ARCH, "-o", tmp, *objs, "-Xcompiler", "-fopenmp", "-lgomp"],
             verbose)
        os.replace(tmp, LIB)
        with open(stamp_file, "w") as f:
            f.write(stamp)
    cli_src = os.path.join(CSRC, "spinwalk_cli.cpp")
    if force or not os.path.exists(CLI) or os.path.getmtime(CLI) < max(
            os.path.getmtime(LIB), os.path.getmtime(cli_src)):
        _run(["g++", "-O2", "-std=c++17", f"-I{INC}", cli_src, "-o", CLI, f"-L{PKG}",
              "-lspinwalk_gpu", "-Wl,-rpath,$ORIGIN"], verbose)
    return LIB


def build_oracle(verbose=False):
    od = os.path.join(ROOT, "oracle")
    _run(["make", "-s", "-C", od, "liboracle.so", "libsynth.so"], verbose)
    if REF_TREE and os.path.isdir(os.path.join(REF_TREE, "src", "sim")):
        _run(["make", "-s", "-C", od, "ref", f"REF={REF_TREE}"], verbose)


def build_all(verbose=False, force=False):
    with ThreadPoolExecutor(max_workers=2) as ex:
        f1 = ex.submit(build_lib, verbose, force)
        f2 = ex.submit(build_oracle, verbose)
        f1.result()
        f2.result()


if __name__ == "__main__":
    build_all(verbose=True, force="--force" in sys.argv)
