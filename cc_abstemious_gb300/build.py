"""Build recipe for libbem_gb300.so (in-tree, sm_103a only).

Each translation unit under csrc/ is compiled by nvcc in parallel, then linked
into cc_abstemious_gb300/libbem_gb300.so.  Object files go to
cc_abstemious_gb300/_build/.  No cmake: one -gencode, a few translation units.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libbem_gb300.so")
CLI = os.path.join(HERE, "bem")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")
# host code without fused multiply-adds, so that it gives the same results on
# x86-64 and aarch64 (gcc contracts a * b + c by default where FMA is baseline)
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
          "-Xcompiler", "-ffp-contract=off", "-I", os.path.join(ROOT, "include")]


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _headers_mtime():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(ROOT, "include", "bem.h"))
    return max(os.path.getmtime(h) for h in hs)


def _compile(src, verbose, extra):
    out = os.path.join(OBJ, src + ".o")
    path = os.path.join(CSRC, src)
    if os.path.exists(out) and os.path.getmtime(out) >= max(os.path.getmtime(path), _headers_mtime()):
        return out
    cmd = [NVCC] + ARCH + COMMON + extra + ["-c", path, "-o", out]
    if src.endswith(".cu"):
        cmd += ["-Xptxas", "-v"] if os.environ.get("BEM_PTXAS_V") else []
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
    if r.stderr and (verbose or os.environ.get("BEM_PTXAS_V")):
        sys.stderr.write(r.stderr)
    return out


def build(force=False, verbose=False, extra=()):
    os.makedirs(OBJ, exist_ok=True)
    srcs = sources()
    if force:
        for s in srcs:
            o = os.path.join(OBJ, s + ".o")
            if os.path.exists(o):
                os.remove(o)
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose, list(extra)), srcs))
    if not (os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(o) for o in objs)):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
        os.replace(LIB + ".tmp", LIB)
    build_cli(verbose)
    return LIB


def build_cli(verbose=False):
    """The `bem input.json` program (cli/bem_main.cpp), linked against the
    library in this directory (rpath $ORIGIN)."""
    src = os.path.join(HERE, "cli", "bem_main.cpp")
    if os.path.exists(CLI) and os.path.getmtime(CLI) >= max(os.path.getmtime(src), os.path.getmtime(LIB)):
        return CLI
    cxx = os.environ.get("CXX", "g++")
    cmd = [cxx, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), src, "-o", CLI + ".tmp",
           "-L", HERE, "-l:libbem_gb300.so", "-Wl,-rpath,$ORIGIN"]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.run(cmd, check=True)
    os.replace(CLI + ".tmp", CLI)
    return CLI


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
