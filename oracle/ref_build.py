"""ORACLE recipe (test infrastructure only): compiles the reference's own HLSL
compute shaders as C++ into oracle/_ref/libvlt_ref.so.

The reference's lighting back end is HLSL (shader/restir/*.hlsl, shader/denoise/*.hlsl
and their includes), normally compiled by DXC and run through Vulkan. This recipe
reads those files where they lie in the reference tree, applies the textual rewrites
listed in REWRITES (HLSL syntax that C++ spells differently; nothing in the
algorithms is touched), writes the rewritten copies to oracle/_ref/gen/shader/ and
compiles them with g++ against oracle/hlsl/hlsl.hpp (the HLSL vocabulary in C++) and
the per-pass harnesses in oracle/hlsl/passes/ (bindings, push constants, dispatch).
Nothing from the reference tree is copied into the repository: oracle/_ref/ is
build output, ignored by git.

The reference tree is looked up in $VLT_REFERENCE_ROOT, else ../reference next to the
repository's parent (the layout of the build container). Where it is absent (the GPU
machines), build() returns None and the tests that need it are skipped; the golden
fixtures made from it (tests/golden/) stand in there.
"""
import itertools
import os
import re
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
GEN = os.path.join(OUT_DIR, "gen")
LIB = os.path.join(OUT_DIR, "libvlt_ref.so")
HARNESS_DIR = os.path.join(HERE, "hlsl", "passes")
SHIM = [os.path.join(HERE, "hlsl", "hlsl.hpp"), os.path.join(HERE, "omath.hpp")]
FLAGS = ["-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-w"]


def reference_root():
    env = os.environ.get("VLT_REFERENCE_ROOT")
    cands = [env] if env else []
    cands.append(os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))
    for c in cands:
        if c and os.path.isdir(os.path.join(c, "shader", "restir")):
            return c
    return None


# ------------------------------------------------------------------ rewrites
# Each rewrite: (name, regex, replacement). Applied in order to every shader file.
FLOAT_LIT = r"(?<![\w.])((?:\d+\.\d*|\.\d+)(?:[eE][+-]?\d+)?|\d+[eE][+-]?\d+)"


def _splat(m):
    n = len(m.group(2))
    return "hlsl::splat<%d>(%s)" % (n, m.group(1))


REWRITES = [
    # `(0.04f).xxx`: replicate swizzle of a parenthesised expression.
    ("parenthesised swizzle", re.compile(r"\(([^()]+)\)\.(xx|xxx|xxxx|rr|rrr|rrrr)\b"),
     lambda m: "hlsl::splat<%d>((%s))" % (len(m.group(2)), m.group(1))),
    # `0.5f.xx`, `f90.xxx`: replicate swizzles of scalars (and of vectors' x).
    ("scalar swizzle", re.compile(r"((?:\d+\.\d*f?)|(?:[A-Za-z_]\w*(?:\.[A-Za-z_]\w*)*))\.(xx|xxx|xxxx|rr|rrr|rrrr)\b"),
     _splat),
    # `inout T name` / `out T name` parameters become references.
    ("out parameters", re.compile(r"\b(?:inout|out)\s+([A-Za-z_][\w:]*(?:<[^<>]*>)?)\s+(\w+)"), r"\1& \2"),
    # `in T name` parameters.
    ("in parameters", re.compile(r"([(,]\s*)in\s+([A-Za-z_])"), r"\1\2"),
    # [numthreads(X, Y, Z)] becomes a constant the harness reads.
    ("numthreads", re.compile(r"\[numthreads\(([^)]*)\)\]"), r"static constexpr unsigned hlsl_numthreads[3] = {\1};"),
    # Loop and branch attributes.
    ("control attributes", re.compile(r"\[(?:unroll|loop|branch|flatten|fastopt|allow_uav_condition|call|forcecase)"
                                      r"(?:\([^)]*\))?\]"), ""),
    # Parameter semantics (`: SV_DispatchThreadID`).
    ("semantics", re.compile(r"\s*:\s*SV_\w+"), ""),
    # `#pragma pack_matrix(...)`: matrices are filled from column-major memory.
    ("pack_matrix", re.compile(r"#pragma\s+pack_matrix\([^)]*\)"), ""),
    # `const` locals of struct type: HLSL calls member functions on them freely (C++
    # would need const member functions); the qualifier only guards against writes.
    ("const struct locals", re.compile(r"\bconst\s+(?=[A-Z]\w*\s+\w+\s*=)"), ""),
    # `this` is a value in HLSL.
    ("this", re.compile(r"\bthis\b"), "(*this)"),
    # `(StructType)0`: a zero-initialised struct.
    ("zero struct cast", re.compile(r"\(\s*([A-Za-z_]\w*)\s*\)\s*0\b(?!\.)"), r"\1{}"),
    # Functional scalar casts `uint(x)` etc. (HLSL conversion rules).
    ("scalar casts", re.compile(r"(?<![\w.])(uint|int|float|bool)\s*\("), r"hlsl::cast<\1>("),
    # Unsuffixed floating literals are literal floats.
    ("float literals", re.compile(FLOAT_LIT + r"(?![\w.])"), r"hlsl::lit(\1)"),
]

MAIN_RE = re.compile(r"void\s+main\s*\(([^)]*)\)")
PARAM_RE = re.compile(r"^\s*([A-Za-z_]\w*)\s+(\w+)\s*:\s*(SV_\w+)\s*$")
SEMANTIC_FIELD = {"SV_DispatchThreadID": "dispatch_thread_id", "SV_GroupID": "group_id",
                  "SV_GroupThreadID": "group_thread_id", "SV_GroupIndex": "group_index"}


def strip_comments(text):
    """Comments removed (line structure kept), so that the rewrites see code only."""
    out, i, n = [], 0, len(text)
    while i < n:
        if text.startswith("//", i):
            j = text.find("\n", i)
            i = n if j < 0 else j
        elif text.startswith("/*", i):
            j = text.find("*/", i + 2)
            j = n if j < 0 else j + 2
            out.append("\n" * text.count("\n", i, j))
            i = j
        else:
            out.append(text[i])
            i += 1
    return "".join(out)


VEC_CTOR = re.compile(r"(?<![\w.])((?:float|int|uint|bool|half)[234](?:x[234])?)\s*\(")


def brace_constructors(text):
    """`float2(a, b)` -> `float2{a, b}`: C++ leaves the evaluation order of function
    arguments unspecified (g++ often goes right to left), HLSL evaluates them left to
    right, and `float2(lcg_rand(s), lcg_rand(s))` depends on it; a braced initializer
    list is evaluated left to right."""
    out, pos = [], 0
    while True:
        m = VEC_CTOR.search(text, pos)
        if not m:
            out.append(text[pos:])
            return "".join(out)
        depth, j = 1, m.end()
        while depth and j < len(text):
            depth += {"(": 1, ")": -1}.get(text[j], 0)
            j += 1
        inner = brace_constructors(text[m.end():j - 1])
        out.append(text[pos:m.start()] + m.group(1) + "{" + inner + "}")
        pos = j


def rewrite(text):
    text = strip_comments(text)
    text = brace_constructors(text)
    entry = None
    m = MAIN_RE.search(text)
    if m:
        args = []
        for p in m.group(1).split(","):
            pm = PARAM_RE.match(p)
            if not p.strip():
                continue
            if not pm or pm.group(3) not in SEMANTIC_FIELD:
                args = None  # not a compute entry point (ray-tracing stages); no dispatch wrapper
                break
            args.append("hlsl::thread_param<%s>(t.%s)" % (pm.group(1), SEMANTIC_FIELD[pm.group(3)]))
        if args is not None:
            entry = "static void hlsl_entry(const hlsl::ThreadIds& t) { main(%s); }\n" % ", ".join(args)
    for _, rx, rep in REWRITES:
        text = rx.sub(rep, text)
    if entry:
        text += "\n" + entry
    return text


def write_swizzles(path):
    """vstore<T, N>: the vector storage with named components and every swizzle of
    length 2 to 4 over xyzw and rgba (unions over the component array)."""
    lines = ["// Generated by oracle/ref_build.py: vector storage with swizzles.\n"]
    for n in (2, 3, 4):
        xyzw, rgba = "xyzw"[:n], "rgba"[:n]
        lines.append("template <class T>\nstruct vstore<T, %d> {\n  union {\n    T e[%d];\n" % (n, n))
        lines.append("    struct { T %s; };\n" % ", ".join(xyzw))
        lines.append("    struct { T %s; };\n" % ", ".join(rgba))
        for names in (xyzw, rgba):
            for m in (2, 3, 4):
                for combo in itertools.product(range(n), repeat=m):
                    nm = "".join(names[c] for c in combo)
                    lines.append("    swz<T, %d, %s> %s;\n" % (n, ", ".join(str(c) for c in combo), nm))
        lines.append("  };\n};\n")
    with open(path, "w") as f:
        f.writelines(lines)


def generate(ref):
    src = os.path.join(ref, "shader")
    n = 0
    for dirpath, _, files in os.walk(src):
        for fn in files:
            if not fn.endswith(".hlsl"):
                continue
            rel = os.path.relpath(os.path.join(dirpath, fn), src)
            dst = os.path.join(GEN, "shader", rel)
            os.makedirs(os.path.dirname(dst), exist_ok=True)
            with open(os.path.join(dirpath, fn), encoding="utf-8", errors="replace") as f:
                text = f.read()
            out = rewrite(text)
            if not os.path.exists(dst) or open(dst).read() != out:
                with open(dst, "w") as f:
                    f.write(out)
            n += 1
    sw = os.path.join(GEN, "swizzles.inc")
    write_swizzles(sw + ".tmp")
    if not os.path.exists(sw) or open(sw).read() != open(sw + ".tmp").read():
        os.replace(sw + ".tmp", sw)
    else:
        os.remove(sw + ".tmp")
    return n


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(verbose=False, force=False):
    """Builds oracle/_ref/libvlt_ref.so; returns its path, or None without the
    reference tree."""
    ref = reference_root()
    if ref is None:
        return LIB if os.path.exists(LIB) else None
    os.makedirs(GEN, exist_ok=True)
    generate(ref)
    harness = sorted(f for f in os.listdir(HARNESS_DIR) if f.endswith(".cpp"))
    gen_files = []
    for dirpath, _, files in os.walk(GEN):
        gen_files += [os.path.join(dirpath, f) for f in files]
    inc = ["-I", GEN, "-I", os.path.join(GEN, "shader"), "-I", os.path.join(HERE, "hlsl"),
           "-I", os.path.join(os.path.dirname(HERE), "include")]
    cxx = os.environ.get("CXX", "g++")

    def compile_one(fn):
        s = os.path.join(HARNESS_DIR, fn)
        o = os.path.join(OUT_DIR, fn.replace(".cpp", ".o"))
        if force or _newer(o, [s, __file__] + SHIM + gen_files):
            cmd = [cxx] + FLAGS + inc + ["-c", s, "-o", o]
            if verbose:
                print(" ".join(cmd), flush=True)
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError("reference shader build failed for %s:\n%s%s" % (fn, r.stdout, r.stderr[-20000:]))
        return o

    with ThreadPoolExecutor(max_workers=max(1, min(len(harness), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(compile_one, harness))
    if force or _newer(LIB, objs):
        cmd = [cxx] + FLAGS + ["-shared"] + objs + ["-o", LIB]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("reference shader link failed:\n%s%s" % (r.stdout, r.stderr))
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
