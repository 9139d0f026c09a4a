"""Build the GB300 C-ABI library libcstone_gb300.so in-tree with nvcc (sm_103a only).

Each translation unit under csrc/ is compiled in parallel to an object file under csrc/_build/ and linked with
nvcc -shared. Rebuilds only what changed (source or header newer than its object, or other compiler flags).
CSTONE_GB300_NVCC_FLAGS adds flags to every compile (e.g. "-DNBG_MIN_BLOCKS=8" to trade registers of the neighbour
search for occupancy).
"""
import concurrent.futures as cf
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ_DIR = os.path.join(CSRC, "_build")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
LIB = os.path.join(HERE, "cstone_gb300", "libcstone_gb300.so")

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--extended-lambda", "-Xcompiler", "-fPIC", "-I", INCLUDE,
         "-Xptxas", "-warn-spills"] + os.environ.get("CSTONE_GB300_NVCC_FLAGS", "").split()
STAMP = os.path.join(OBJ_DIR, "flags.txt")


def _headers():
    hs = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))
    return max((os.path.getmtime(h) for h in hs), default=0.0)


def _compile(src, hdr_time, verbose):
    obj = os.path.join(OBJ_DIR, os.path.basename(src) + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), hdr_time):
        return obj, None
    cmd = [NVCC, *ARCH, *FLAGS, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if verbose and (r.stdout or r.stderr):
        sys.stderr.write(r.stdout + r.stderr)
    if r.returncode != 0:
        return obj, f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}"
    return obj, None


def build(verbose=False, jobs=None):
    os.makedirs(OBJ_DIR, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    hdr_time = _headers()
    stamp = " ".join(ARCH + FLAGS)
    if not os.path.exists(STAMP) or open(STAMP).read() != stamp:
        for o in glob.glob(os.path.join(OBJ_DIR, "*.o")):
            os.remove(o)
        with open(STAMP, "w") as f:
            f.write(stamp)
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        results = list(ex.map(lambda s: _compile(s, hdr_time, verbose), srcs))
    errs = [e for _, e in results if e]
    if errs:
        raise RuntimeError("\n".join(errs))
    objs = [o for o, _ in results]
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [NVCC, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


BASELINE_SRC = os.path.join(HERE, "baseline", "cub_sort.cu")
BASELINE_LIB = os.path.join(HERE, "baseline", "libcub_sort.so")


def build_baseline():
    """the CUB sort the reference calls, as a separate library for the benchmark's comparison leg (not the product)"""
    if os.path.exists(BASELINE_LIB) and os.path.getmtime(BASELINE_LIB) >= os.path.getmtime(BASELINE_SRC):
        return BASELINE_LIB
    cmd = [NVCC, *ARCH, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", BASELINE_SRC, "-o", BASELINE_LIB]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"baseline build failed:\n{r.stdout}\n{r.stderr}")
    return BASELINE_LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
