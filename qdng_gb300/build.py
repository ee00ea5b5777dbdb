"""Build libqdg.so in-tree with nvcc for sm_103a (GB300).

    python -m qdng_gb300.build [--verbose]

Translation units are compiled in parallel and linked into
qdng_gb300/libqdg.so; the object files go to qdng_gb300/_build/.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libqdg.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["qdg_kernels.cu", "qdg_persistent.cu", "qdg_api.cu", "qdg_noalloc.cu", "qdg_ensemble.cu",
           "qdg_host.cpp", "qdg_schedule.cpp",
           # the persistent Chebyshev step kernel, one unit per bulk type and grid rank
           "qdg_step_f64_1.cu", "qdg_step_f64_2.cu", "qdg_step_f64_34.cu", "qdg_step_df_2.cu",
           "qdg_step_df_34.cu", "qdg_step_f32_1.cu", "qdg_step_f32_2.cu", "qdg_step_f32_34.cu",
           # one 1-D line on a thread-block cluster
           "qdg_step_cluster.cu", "qdg_step_line64.cu",
           # expectation values of filter operators
           "qdg_filters.cu",
           # the autocorrelation eigen driver
           "qdg_eigen_ac.cu", "qdg_fdkin.cu"]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libqdg.so")
    return exe


def _compile(src, verbose):
    obj = os.path.join(BUILD, src + ".o")
    path = os.path.join(CSRC, src)
    cmd = [nvcc(), "-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
           "-I", os.path.join(HERE, "..", "include"), "-c", path, "-o", obj]
    if src.endswith(".cu"):
        cmd[1:1] = ARCH + ["--expt-relaxed-constexpr"]
        if verbose:
            cmd += ["-Xptxas", "-v"]
    else:
        cmd[1:1] = ["-x", "c++"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(HERE, "..", "include", "qdg.h")]
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    cmd = [nvcc(), "-shared"] + ARCH + objs + ["-o", tmp, "-lcudart", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose="--verbose" in sys.argv))
