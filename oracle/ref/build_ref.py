"""Recipe: compile the reference's own ray-tracing shaders as host code.

TEST INFRASTRUCTURE ONLY. Reads the GLSL where it lies in the reference
checkout (shaders/src of hala-pathtracer), and compiles it with g++ through
oracle/ref/glsl_shim.h and the pipeline stand-in oracle/ref/ref_harness.inl,
one shared library per feature permutation, into oracle/_ref/. Nothing of the
reference is written anywhere: the assembled translation unit goes to the
compiler on standard input.

Mechanical steps applied to the GLSL text (everything else is compiled as
written):
  * `#include` is resolved like the reference's shader build (relative to the
    including file, then shaders/src), each file once; the descriptor-layout
    include hala-pathtracer/inc/global.glsl is replaced by
    oracle/ref/global_binding.h (the same names as host objects);
  * `#version`, `#extension` and `precision` lines are dropped; comments are
    stripped;
  * parameter qualifiers: `in T x` -> `T x`, `out/inout T x` -> `T& x`;
  * decimal literals get an `f` suffix (GLSL literals are single precision);
  * the two buffer_reference blocks of inc/types.glsl become structs holding
    a pointer (`Vertices`, `Indices`);
  * each shader's `main` is renamed <file>_main;
  * a call with two or more arguments that draw from the RNG (only
    pathtracer.rgen.glsl:186) gets its arguments evaluated through a braced
    tuple, because GLSL evaluates arguments left to right and C++ does not
    specify the order.
The feature macros are the reference's: ROUGHNESS_REGULARIZE_EVAL always
(shaders/src/make_shaders.yaml:3-4), USE_<NAME> per optional macro
(shaders/build.rs:89-93).
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(os.path.dirname(HERE), "_ref")
DEFAULT_SRC = os.path.join(os.environ.get("HALA_REFERENCE", "/root/reference"), "shaders", "src")

SHADERS = [
    "hala-pathtracer/pathtracer.rgen.glsl",
    "hala-pathtracer/perspective_ray.rcall.glsl",
    "hala-pathtracer/orthographic_ray.rcall.glsl",
    "hala-pathtracer/env_sky_eval.rcall.glsl",
    "hala-pathtracer/env_sky_sample.rcall.glsl",
    "hala-pathtracer/env_map_eval.rcall.glsl",
    "hala-pathtracer/env_map_sample.rcall.glsl",
    "hala-pathtracer/point_light_sample.rcall.glsl",
    "hala-pathtracer/directional_light_sample.rcall.glsl",
    "hala-pathtracer/spot_light_sample.rcall.glsl",
    "hala-pathtracer/quad_light_sample.rcall.glsl",
    "hala-pathtracer/sphere_light_sample.rcall.glsl",
    "hala-pathtracer/diffuse_bxdf_eval.rcall.glsl",
    "hala-pathtracer/diffuse_bxdf_sample.rcall.glsl",
    "hala-pathtracer/disney_bxdf_eval.rcall.glsl",
    "hala-pathtracer/disney_bxdf_sample.rcall.glsl",
    "hala-pathtracer/triangles.rchit.glsl",
    "hala-pathtracer/lights.rint.glsl",
    "hala-pathtracer/lights.rchit.glsl",
    "hala-pathtracer/pathtracer.rmiss.glsl",
    "hala-pathtracer/shadow_ray.rmiss.glsl",
]

# Feature permutations the reference host selects (src/bin/hala-pathtracer.rs:101-114).
PERMUTATIONS = {
    "base": ["PATH_TRACER"],
    "transparent": ["PATH_TRACER", "TRANSPARENT"],
    "medium": ["PATH_TRACER", "MEDIUM", "VOL_MIS"],
    "medium_transparent": ["PATH_TRACER", "MEDIUM", "VOL_MIS", "TRANSPARENT"],
}

_LIT = re.compile(r"(?<![\w.])((?:\d+\.\d*|\.\d+)(?:[eE][+-]?\d+)?|\d+[eE][+-]?\d+)(?![\w.])")


def _strip_comments(text):
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    return re.sub(r"//[^\n]*", "", text)


def _split_args(s):
    parts, depth, cur = [], 0, []
    for ch in s:
        if ch in "([{":
            depth += 1
        elif ch in ")]}":
            depth -= 1
        if ch == "," and depth == 0:
            parts.append("".join(cur))
            cur = []
        else:
            cur.append(ch)
    parts.append("".join(cur))
    return parts


def _sequence_rng_calls(text):
    """f(a, rand(r), rand(r)) -> std::apply(f, std::tuple{a, rand(r), rand(r)})."""
    out, i = [], 0
    pat = re.compile(r"\b([A-Za-z_]\w*)\s*\(")
    while True:
        m = pat.search(text, i)
        if not m:
            out.append(text[i:])
            return "".join(out)
        depth, j = 1, m.end()
        while j < len(text) and depth:
            depth += {"(": 1, ")": -1}.get(text[j], 0)
            j += 1
        args = text[m.end():j - 1]
        if sum(1 for a in _split_args(args) if re.search(r"\brand\d?\s*\(", a)) >= 2:
            out.append(text[i:m.start()])
            out.append(f"std::apply([&](auto... a_) {{ return {m.group(1)}(a_...); }}, std::tuple{{{args}}})")
            i = j
        else:
            out.append(text[i:m.end()])
            i = m.end()


def _transform(text):
    text = re.sub(r"\b(inout|out)\s+(\w+)\s+(\w+)", r"\2& \3", text)
    text = re.sub(r"\bin\s+(\w+)\s+(\w+)", r"\1 \2", text)
    text = _LIT.sub(lambda m: m.group(1) + "f", text)
    text = _sequence_rng_calls(text)
    text = re.sub(r"readonly\s+buffer\s+(\w+)\s*\{\s*(\w+)\s+data\s*\[\s*\]\s*;\s*\}\s*;",
                  r"struct \1 { const \2* data; };", text)
    return text


def _inline(path, src_root, seen, out):
    key = os.path.normpath(path)
    if key in seen:
        return
    seen.add(key)
    rel = os.path.relpath(key, src_root).replace(os.sep, "/")
    if rel == "hala-pathtracer/inc/global.glsl":
        out.append('#include "global_binding.h"\n')
        return
    with open(key) as f:
        lines = f.read().split("\n")
    buf = []
    for line in lines:
        s = line.strip()
        m = re.match(r'#\s*include\s+"([^"]+)"', s)
        if m:
            out.append(_transform(_strip_comments("\n".join(buf))) + "\n")
            buf = []
            inc = m.group(1)
            cand = os.path.join(os.path.dirname(key), inc)
            if not os.path.exists(cand):
                cand = os.path.join(src_root, inc)
            _inline(cand, src_root, seen, out)
            continue
        if s.startswith("#version") or s.startswith("#extension") or s.startswith("precision "):
            continue
        buf.append(line)
    out.append(_transform(_strip_comments("\n".join(buf))) + "\n")


def assemble(src_root, macros):
    out = ['#include "glsl_shim.h"\n', "#define ROUGHNESS_REGULARIZE_EVAL 1\n"]
    out += [f"#define USE_{m} 1\n" for m in macros]
    seen = set()
    for sh in SHADERS:
        name = os.path.basename(sh).replace(".glsl", "").replace(".", "_")
        out.append(f"#define main {name}_main\n")
        _inline(os.path.join(src_root, sh), src_root, seen, out)
        out.append("#undef main\n")
    out.append('#include "ref_harness.inl"\n')
    return "".join(out)


def lib_path(perm):
    return os.path.join(OUT, f"libhala_ref_{perm}.so")


def build(src_root=None, perms=None, force=False):
    """Builds oracle/_ref/libhala_ref_<perm>.so; returns {perm: path}.
    Returns {} when the reference checkout is not present."""
    src_root = src_root or os.environ.get("HALA_REFERENCE_SHADERS", DEFAULT_SRC)
    if not os.path.isdir(src_root):
        return {}
    os.makedirs(OUT, exist_ok=True)
    deps = [os.path.join(HERE, f) for f in ("glsl_shim.h", "global_binding.h", "ref_harness.inl", "build_ref.py")]
    deps.append(os.path.join(os.path.dirname(HERE), "pmath.h"))
    res = {}
    for perm in (perms or PERMUTATIONS):
        path = lib_path(perm)
        if not force and os.path.exists(path) and all(os.path.getmtime(d) <= os.path.getmtime(path) for d in deps):
            res[perm] = path
            continue
        tu = assemble(src_root, PERMUTATIONS[perm])
        import platform
        isa = ["-mfma"] if platform.machine() in ("x86_64", "AMD64") else []
        cmd = ["g++", "-std=c++20", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread",
               "-w", "-I", HERE] + isa + ["-x", "c++", "-", "-o", path + ".tmp"]
        r = subprocess.run(cmd, input=tu, text=True, capture_output=True)
        if r.returncode != 0:
            raise RuntimeError(f"compiling the reference shaders ({perm}) failed:\n{r.stderr[:6000]}")
        os.replace(path + ".tmp", path)
        res[perm] = path
    return res


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
