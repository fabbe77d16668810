"""Build recipe for libgbmg.so (the CUDA kernels + C ABI), sm_103a only.

Each .cu translation unit is compiled in parallel with nvcc, then linked into
fortrancfd_gb300/_build/libgbmg.so.  The library is built in-tree (never
installed) so that the process that uses it loads it from the package.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
BUILD = os.path.join(HERE, "_build")
SO = os.path.join(BUILD, "libgbmg.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-I", CSRC, "-I", INCLUDE]
# Translation units whose FP64 results must equal the oracle's bit for bit are
# compiled without multiply-add contraction.
FILE_FLAGS = {"momentum.cu": ["-fmad=false"], "ccd.cu": ["-fmad=false"]}


def nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _stale():
    if not os.path.exists(SO):
        return True
    t = os.path.getmtime(SO)
    deps = sources() + [os.path.join(CSRC, f) for f in os.listdir(CSRC)
                        if f.endswith((".h", ".cuh"))] + [os.path.join(INCLUDE, "gbmg.h")]
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return SO
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()
    objs = [os.path.join(BUILD, os.path.basename(s)[:-3] + ".o") for s in srcs]

    def compile_one(pair):
        src, obj = pair
        cmd = [nvcc(), *ARCH, *FLAGS, *FILE_FLAGS.get(os.path.basename(src), []), "-c", src,
               "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        return src, r

    with ThreadPoolExecutor(max_workers=max(1, len(srcs))) as ex:
        for src, r in ex.map(compile_one, zip(srcs, objs)):
            if verbose and r.stderr:
                sys.stderr.write(r.stderr)
            if r.returncode != 0:
                sys.stderr.write(r.stdout + r.stderr)
                raise RuntimeError(f"nvcc failed on {os.path.basename(src)}")
    tmp = SO + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("link of libgbmg.so failed")
    os.replace(tmp, SO)
    return SO


if __name__ == "__main__":
    print(build(force=True, verbose="-v" in sys.argv))
