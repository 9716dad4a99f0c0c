"""Builds libfvgb.so in-tree: every csrc/*.cu and csrc/*.cpp compiled for
sm_103a with nvcc (translation units in parallel), linked as one shared
library next to this file; then the headless driver fvgb_run
(csrc/driver/fvgb_run.cpp, host C++ over the C ABI) next to it."""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libfvgb.so")
DRIVER_SRC = os.path.join(CSRC, "driver", "fvgb_run.cpp")
DRIVER = os.path.join(HERE, "fvgb_run")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _stale(lib, deps):
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    os.makedirs(OBJ, exist_ok=True)
    srcs = sources()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "fvgb.h"))
    if not force and not _stale(LIB, srcs + headers + [__file__]):
        build_driver(force)
        return LIB
    # -ffp-contract=off: host arithmetic (layout coefficients, forces) rounds the same on x86 and Arm
    common = [nvcc(), "-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "-I", os.path.join(ROOT, "include"), "-I", CSRC] + ARCH
    if os.environ.get("FVGB_PTXAS_VERBOSE"):
        common += ["-Xptxas", "-v"]
    # extra nvcc flags, e.g. -DFVGB_SOFT_MUL=0 (plain products on the FP64 pipe, for side-by-side timing)
    common += os.environ.get("FVGB_NVCC_EXTRA", "").split()

    def compile_one(src):
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        cmd = common + ["-x", "cu" if src.endswith(".cu") else "c++", "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), "-shared"] + ARCH + objs + ["-o", tmp, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    build_driver(True)
    return LIB


def build_driver(force=False):
    """fvgb_run: the driver loop over the C ABI, linked against libfvgb.so (rpath $ORIGIN)."""
    header = os.path.join(ROOT, "include", "fvgb.h")
    if not force and not _stale(DRIVER, [DRIVER_SRC, header, LIB]):
        return DRIVER
    cxx = os.environ.get("CXX", "g++")
    tmp = DRIVER + ".tmp"
    cmd = [cxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), DRIVER_SRC, "-o", tmp,
           "-L", HERE, "-lfvgb", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"driver build failed:\n{r.stderr}")
    os.replace(tmp, DRIVER)
    return DRIVER


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
