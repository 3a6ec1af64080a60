"""Build recipe of libhalapt.so (the CUDA library behind include/hala_pt.h).

Compiles every csrc/*.cu for sm_103a only, one translation unit per process,
and links them into csrc/../_build/libhalapt.so. No cmake; nvcc only.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libhalapt.so")
INCLUDE = os.path.join(HERE, "..", "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off", "-I", CSRC, "-I", INCLUDE]


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs + [os.path.join(INCLUDE, "hala_pt.h")]


# Shading code is compiled without multiply-add contraction so it rounds like
# the CPU oracle (explicit fmaf calls are still fused).
PER_FILE_FLAGS = {f: ["-fmad=false"] for f in ("pt_render.cu", "pt_shade_plain.cu", "pt_shade_medium.cu",
                                                "pt_shade_cache.cu", "pt_shade_multi.cu", "pt_shade_multi_medium.cu")}


def _compile(src, verbose_ptxas=False):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    extra = PER_FILE_FLAGS.get(os.path.basename(src), [])
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + extra + (["-Xptxas", "-v"] if verbose_ptxas else []) + \
        ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    return obj, r.stderr


def build(force=False, verbose_ptxas=False):
    """Builds libhalapt.so if any source or header is newer; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()
    if not force and not verbose_ptxas and os.path.exists(LIB):
        mt = os.path.getmtime(LIB)
        if all(os.path.getmtime(f) <= mt for f in srcs + headers() + [__file__]):
            return LIB
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose_ptxas), srcs))
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose_ptxas:
        return LIB, "\n".join(e for _, e in results)
    return LIB


if __name__ == "__main__":
    import sys
    out = build(force=True, verbose_ptxas="-v" in sys.argv)
    if isinstance(out, tuple):
        print(out[1])
        out = out[0]
    print(out)
