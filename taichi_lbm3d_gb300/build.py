"""Build liblbm_gb300.so in-tree with nvcc for sm_103a (GB300) only.

Each .cu under csrc/ is compiled to an object in parallel, then linked into
taichi_lbm3d_gb300/liblbm_gb300.so.  Flags:
  -gencode arch=compute_103a,code=sm_103a   the only target
  -fmad=false / -ffp-contract=off           no multiply-add fusion beyond the
                                            explicit lbm_fma() calls, so the FP32
                                            kernels keep the reference's rounding
"""
import concurrent.futures as cf
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "liblbm_gb300.so")
INCLUDE = os.path.join(os.path.dirname(PKG), "include")

NVCC_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-O3", "-lineinfo", "-std=c++17", "-fmad=false",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-O2",
]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, verbose=False):
    obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
    if not _stale(obj, [src] + _headers()):
        return obj, ""
    cmd = [_nvcc()] + NVCC_FLAGS + _extra_flags() + ["-Xptxas", "-v", "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr[-4000:]))
    return obj, r.stderr


def _extra_flags():
    """Extra nvcc flags from LBM_NVCC_EXTRA (e.g. "-DLBM_SP_MINBLOCKS=6") for tuning builds."""
    return os.environ.get("LBM_NVCC_EXTRA", "").split()


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()
    stamp = os.path.join(BUILD, "flags.txt")
    flags = " ".join(NVCC_FLAGS + _extra_flags())
    if not os.path.exists(stamp) or open(stamp).read() != flags:
        force = True
    if force:
        for f in os.listdir(BUILD):
            os.remove(os.path.join(BUILD, f))
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), srcs))
    objs = [o for o, _ in results]
    if verbose:
        for _, log in results:
            if log:
                sys.stderr.write(log)
    if force or _stale(LIB, objs):
        tmp = LIB + ".tmp"
        cmd = [_nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-shared", "-o", tmp] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s" % r.stderr[-4000:])
        os.replace(tmp, LIB)
    with open(stamp, "w") as fh:
        fh.write(flags)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
