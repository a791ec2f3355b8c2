"""Builds libshll_gb300.so (the CUDA kernels and the C-ABI of include/shll.h) for sm_103a.

Each translation unit is compiled by its own nvcc process (in parallel), then linked with
nvcc -shared.  Output: <package>/_build/libshll_gb300.so (git-ignored, rebuilt on each machine).
"""
import concurrent.futures
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libshll_gb300.so")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", CSRC]
# translation units and their extra flags: -fmad=false where results must not depend on the
# compiler's choice of fused multiply-adds (bit-exact reference arithmetic; the mixed engine,
# whose halo recomputation must agree bit for bit with each cell's owner)
UNITS = {
    "capi.cu": [],
    "plain_fast.cu": [],
    "plain_exact.cu": ["-fmad=false"],
    "mixed1d.cu": ["-fmad=false"],
    "mixed2d.cu": ["-fmad=false"],
    "reduce.cu": [],
    "plain_batch.cu": [],
    "plain_batch_exact.cu": ["-fmad=false"],
    "refglobals.cu": [],
}
HEADERS = ["shll_internal.h", "shll_plain.cuh", "mixed.h", "mixed_common.cuh", "plain_batch.h",
           "plain_batch_kernels.cuh"]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(unit, flags, verbose):
    src = os.path.join(CSRC, unit)
    obj = os.path.join(BUILD, unit.replace(".cu", ".o"))
    deps = [src] + [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(HERE, "..", "include", "shll.h")]
    if not _stale(obj, deps):
        return obj, ""
    cmd = [NVCC] + COMMON + flags + ["-c", src, "-o", obj]
    if verbose:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {unit}:\n{r.stderr}")
    return obj, r.stderr


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        futs = [ex.submit(_compile, u, f, verbose) for u, f in UNITS.items()]
        objs = []
        for fu in futs:
            obj, log = fu.result()
            objs.append(obj)
            if verbose and log:
                print(log, file=sys.stderr)
    if _stale(LIB, objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
    inc = ["-I", os.path.join(HERE, "..", "include")]
    link = ["-L", BUILD, f"-Wl,-rpath,{BUILD}"]
    # the reference-style C driver (host code in C over the C-ABI)
    drv = os.path.join(BUILD, "shll_tube")
    src = os.path.join(HERE, "host", "shll_tube.c")
    if _stale(drv, [src, LIB]):
        cmd = ["gcc", "-O2", "-Wall"] + inc + [src, "-o", drv] + link + ["-lshll_gb300"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"driver build failed:\n{r.stderr}")
    # a reference-style program whose main() is unchanged: it takes the stage functions from the
    # library, which reads its problem constants and sets its DT
    drv = os.path.join(BUILD, "shll_ref_main")
    src = os.path.join(HERE, "host", "shll_ref_main.c")
    if _stale(drv, [src, LIB]):
        cmd = ["gcc", "-O2", "-Wall"] + inc + [src, "-o", drv] + link + ["-lshll_gb300"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference-style program build failed:\n{r.stderr}")
    # team-aware stages (OpenMP, base-omp's calling pattern) and their driver; skipped with a
    # message where the C compiler has no OpenMP
    omp_lib = os.path.join(BUILD, "libshll_gb300_omp.so")
    omp_drv = os.path.join(BUILD, "shll_omp")
    omp_src = os.path.join(HERE, "host", "shll_omp_stages.c")
    drv_src = os.path.join(HERE, "host", "shll_omp.c")
    if _stale(omp_lib, [omp_src, LIB]) or _stale(omp_drv, [drv_src, omp_src, LIB]):
        cmds = [["gcc", "-O2", "-Wall", "-fopenmp", "-shared", "-fPIC"] + inc + [omp_src, "-o", omp_lib] + link
                + ["-lshll_gb300"],
                ["gcc", "-O2", "-Wall", "-fopenmp"] + inc + [drv_src, "-o", omp_drv] + link
                + ["-lshll_gb300_omp", "-lshll_gb300"]]
        for cmd in cmds:
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                print(f"OpenMP driver not built (gcc -fopenmp failed):\n{r.stderr}", file=sys.stderr)
                break
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
