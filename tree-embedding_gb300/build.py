"""Build recipe for libtsvd_gb300.so (sm_103a) and the tree_svd CLI.

Every translation unit is compiled by nvcc in parallel (one -gencode, no
cmake); outputs stay in this directory (_build/ and the .so, git-ignored).
"""
import concurrent.futures as cf
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libtsvd_gb300.so")
CLI = os.path.join(HERE, "tree_svd")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

NVCC = os.environ.get("NVCC", "nvcc")


ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-I" + INCLUDE, "-I" + CSRC,
          "-Xcompiler", "-fPIC,-pthread,-ffp-contract=off", "-diag-suppress", "177"]


def _newest(paths):
    return max((os.path.getmtime(p) for p in paths), default=0.0)


def _compile(src, headers_mtime):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), headers_mtime):
        return obj
    cmd = [NVCC] + ARCH + COMMON + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return obj


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    headers = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(INCLUDE, "*.h"))
    hm = _newest(headers)
    with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        objs = list(ex.map(lambda s: _compile(s, hm), srcs))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < _newest(objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-Xcompiler", "-pthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    cli_src = os.path.join(CSRC, "cli", "tree_svd.cpp")
    if os.path.exists(cli_src) and (not os.path.exists(CLI) or
                                    os.path.getmtime(CLI) < max(os.path.getmtime(LIB),
                                                                os.path.getmtime(cli_src))):
        cmd = ["g++", "-O2", "-std=c++17", "-pthread", "-I" + INCLUDE, cli_src, "-o", CLI, "-L" + HERE,
               "-ltsvd_gb300", "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("cli link failed:\n%s%s" % (r.stdout, r.stderr))
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
