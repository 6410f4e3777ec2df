"""Build the engine library foort_gb300/libfoort_gpu.so for sm_103a (GB300).

Every .cu / .cpp under csrc/ is compiled to an object under _build/ (in parallel, only
when stale) and linked into one shared library with a plain C ABI.
"""
import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libfoort_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code is compiled without floating-point contraction so that the host-side camera
# frame is the same on x86-64 and aarch64 hosts.
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
                  "--expt-relaxed-constexpr"]
CXXFLAGS = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _headers():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(CSRC, "*.inc")) + [os.path.join(HERE, "..", "include", "foort_gpu.h")]


def _stale(obj, src, newest_header):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return t < os.path.getmtime(src) or t < newest_header


# The mixed-precision kernels flush FP32 denormals (their FP64 code is unaffected);
# FP32 division stays correctly rounded so that no operation has a systematic bias.
MIXED_FLAGS = ["-ftz=true"]


def _compile(src, obj, extra, verbose):
    if src.endswith(".cu"):
        more = MIXED_FLAGS if os.path.basename(src).startswith("k_mixed_") else []
        cmd = [nvcc()] + NVFLAGS + more + extra + ["-c", src, "-o", obj]
    else:
        cmd = ["g++"] + CXXFLAGS + ["-I" + os.path.join(HERE, "..", "include"), "-I/usr/local/cuda/include",
                                    "-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {src}\n{r.stdout}\n{r.stderr}")
    return r.stderr


def build(force=False, verbose=False, ptxas_info=False, jobs=None):
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    newest = max(os.path.getmtime(h) for h in _headers())
    todo, objs = [], []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s) + ".o")
        objs.append(o)
        if force or _stale(o, s, newest):
            todo.append((s, o))
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    logs = {}
    if todo:
        with ThreadPoolExecutor(max_workers=jobs or min(16, os.cpu_count() or 4)) as ex:
            futs = {ex.submit(_compile, s, o, extra, verbose): s for s, o in todo}
            for f, s in futs.items():
                logs[s] = f.result()
    if todo or not os.path.exists(LIB):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed\n{r.stdout}\n{r.stderr}")
    return logs


if __name__ == "__main__":
    logs = build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv)
    for s, log in logs.items():
        if log.strip():
            print(f"== {os.path.basename(s)}\n{log}")
    print(LIB)
