"""ORACLE — test infrastructure only. Recipe that compiles the reference's DDGI shaders as FP64 C++ so the
oracle restatement can be checked against the reference's own shader code.

It reads the stage sources where they lie under the reference tree (assets/shaders/irradiance_probe_update
.rgen / .rchit / .rmiss and probe_conv.comp; the specular GI pass mirror_reflections.rgen / .rchit / .rmiss;
the RT shadow pass shadow.rgen / .rchit / .rmiss; the deferred pass deferred_tiled.comp from its doLight
function, which holds the DDGI consumer block; with their includes), rewrites the GLSL declarations into
C++ over glsl_shim.hpp (every float becomes a double), keeps only the functions each stage's entry reaches,
and writes the result to oracle/_ref/gen/stages.inc. ref_harness.cpp includes it, supplies traceRayEXT per
pipeline (the oracle's exact FP64 closest hit decides which triangle a ray hits; that pipeline's closest-hit
or miss stage then runs on the payload, as the ray-tracing pipeline would) and exports a small C API.
Everything it writes goes to oracle/_ref/, which is not committed. Machines without the reference sources
build nothing.

The rewrite is mechanical; what it changes, construct by construct:
  #version / #extension                 dropped; #include inlined once per stage
  layout(...) qualifiers                 dropped
  uniform / buffer blocks                a struct type plus one instance; unsized arrays become pointers
  uniform sampler2D / image2D / ...      plain globals of the shim's types (the harness binds them)
  shared (compute shaders)               plain globals
  rayPayloadEXT T p (location L)         a global T p; traceRayEXT(..., L) passes its address to the
                                         pipeline's dispatcher (traceRay_<pipeline> in the harness)
  rayPayloadInEXT T p                    a pointer set by the harness; uses of p read through it
  hitAttributeEXT vec2 bary              a global the harness sets before the closest-hit stage runs
  out / inout parameters                 references
  T x[n] = T[](a, b, ...)                brace initialisers
  floating literals                      read at their decimal value in FP64 (the shader rounds them to
                                         float32; the comparison isolates arithmetic, see the pin test)
  main                                   <stage>::stage_main (a stage entered elsewhere keeps its name)
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
from pathlib import Path

# the reference source tree: ANEREND_REFERENCE when set, else where this build environment mounts it
REFERENCE = Path(os.environ.get("ANEREND_REFERENCE", "/root/reference"))
SHADERS = REFERENCE / "assets" / "shaders"
HERE = Path(__file__).resolve().parent
ORACLE = HERE.parent
OUT = ORACLE / "_ref"
GEN = OUT / "gen"
LIB = OUT / "libddgi_refshader.so"

# the shim's builtins, declared in each stage so they hide the C library's functions of the same names
USING = " ".join(f"using glsl::{f};" for f in (
    "abs", "floor", "fract", "sqrt", "sin", "cos", "acos", "exp", "log", "pow", "max", "min", "mod", "clamp",
    "mix", "dot", "length", "distance", "normalize", "cross", "reflect"))

# stage -> (source, ray-tracing pipeline whose traceRayEXT dispatcher it calls, entry function)
STAGES = {
    "rgen": ("irradiance_probe_update.rgen", "probe", "main"),
    "rchit": ("irradiance_probe_update.rchit", "probe", "main"),
    "rmiss": ("irradiance_probe_update.rmiss", "probe", "main"),
    "conv": ("probe_conv.comp", None, "main"),
    "mrgen": ("mirror_reflections.rgen", "mirror", "main"),
    "mrchit": ("mirror_reflections.rchit", "mirror", "main"),
    "mrmiss": ("mirror_reflections.rmiss", "mirror", "main"),
    "srgen": ("shadow.rgen", "shadow", "main"),
    "srchit": ("shadow.rchit", "shadow", "main"),
    "srmiss": ("shadow.rmiss", "shadow", "main"),
    "deferred": ("deferred_tiled.comp", None, "doLight"),
}


def _inline(path: Path, seen: set) -> str:
    out = []
    for line in path.read_text().splitlines():
        m = re.match(r'\s*#include\s+"([^"]+)"', line)
        if m:
            inc = SHADERS / m.group(1)
            if inc.name not in seen:
                seen.add(inc.name)
                out.append(_inline(inc, seen))
            continue
        if re.match(r"\s*#(version|extension)\b", line):
            continue
        out.append(line)
    return "\n".join(out)


def _strip_comments(src: str) -> str:
    src = re.sub(r"/\*.*?\*/", " ", src, flags=re.S)
    return re.sub(r"//[^\n]*", "", src)


def _items(src: str):
    """Splits a translation unit into top-level items: ('pp', line), ('func', header, body), ('decl', text)."""
    items = []
    i, n = 0, len(src)
    buf = ""
    while i < n:
        c = src[i]
        if not buf.strip() and c == "#":
            j = src.find("\n", i)
            j = n if j < 0 else j
            items.append(("pp", src[i:j].strip()))
            i = j + 1
            buf = ""
            continue
        if c == "{":
            depth, j = 1, i + 1
            while depth and j < n:
                depth += {"{": 1, "}": -1}.get(src[j], 0)
                j += 1
            head = buf.strip()
            body = src[i:j]
            if re.search(r"\)\s*$", head) and not re.match(r"(layout|uniform|buffer|struct)\b", head):
                items.append(("func", head, body))
                buf = ""
                i = j
                continue
            # struct or block: take through the terminating semicolon
            k = src.find(";", j)
            items.append(("decl", (buf + src[i:k + 1]).strip()))
            buf = ""
            i = k + 1
            continue
        if c == ";":
            if buf.strip():
                items.append(("decl", (buf + ";").strip()))
            buf = ""
            i += 1
            continue
        buf += c
        i += 1
    return items


def _func_name(head: str) -> str:
    return re.match(r".*?(\w+)\s*\($", re.sub(r"\(([^()]*)\)\s*$", "(", head), re.S).group(1)


def _params(head: str) -> str:
    m = re.match(r"(.*?\w+\s*)\((.*)\)\s*$", head, re.S)
    ret, params = m.group(1), m.group(2)
    out = []
    for p in [p.strip() for p in params.split(",") if p.strip()]:
        p = re.sub(r"\bin\s+", "", p)
        q = re.match(r"(?:const\s+)?(inout|out)\s+(\w+)\s+(\w+)$", p)
        if q:
            p = f"{q.group(2)}& {q.group(3)}"
        out.append(p)
    return f"{ret}({', '.join(out)})"


def _decl(text: str, stage: str, payloads: dict, inpayload: list) -> str:
    t = re.sub(r"layout\s*\([^)]*\)\s*", "", text).strip()
    t = re.sub(r"\b(readonly|writeonly|restrict|coherent|volatile)\b\s*", "", t)
    t = re.sub(r"^shared\s+", "", t)
    if re.match(r"in\s*;$", t):  # local_size declaration of a compute shader
        return ""
    m = re.match(r"(uniform|buffer)\s+(\w+)\s*(\{.*\})\s*(\w+)\s*;$", t, re.S)
    if m:  # block
        body = re.sub(r"(\w+)\s+(\w+)\s*\[\s*\]\s*;", r"\1* \2 = nullptr;", m.group(3))
        return f"struct {m.group(2)} {body};\n{m.group(2)} {m.group(4)};"
    m = re.match(r"uniform\s+(\w+)\s+(\w+)\s*\[\s*\]\s*;$", t)
    if m:
        return f"{m.group(1)}* {m.group(2)} = nullptr;"
    m = re.match(r"uniform\s+(\w+)\s+(\w+)\s*\[\s*(\d+)\s*\]\s*;$", t)
    if m:
        return f"{m.group(1)} {m.group(2)}[{m.group(3)}];"
    m = re.match(r"uniform\s+(\w+)\s+(\w+)\s*;$", t)
    if m:
        return f"{m.group(1)} {m.group(2)};"
    m = re.match(r"rayPayloadEXT\s+(\w+)\s+(\w+)\s*;$", t)
    if m:
        loc = re.search(r"location\s*=\s*(\d+)", text)
        payloads[int(loc.group(1)) if loc else 0] = m.group(2)
        return f"{m.group(1)} {m.group(2)};"
    m = re.match(r"rayPayloadInEXT\s+(\w+)\s+(\w+)\s*;$", t)
    if m:
        inpayload.append(m.group(2))
        return f"{m.group(1)}* {m.group(2)}__in = nullptr;"
    m = re.match(r"hitAttributeEXT\s+(\w+)\s+(\w+)\s*;$", t)
    if m:
        return f"{m.group(1)} {m.group(2)};"
    # array constructor initialisers: T x[n] = T[](a, b, ...) -> brace initialisers
    return re.sub(r"=\s*\w+\s*\[\s*\d*\s*\]\s*\((.*)\)\s*;$", r"= {\1};", t, flags=re.S)


def translate_stage(stage: str, fname: str, pipeline: str | None = None, entry: str = "main") -> str:
    src = _strip_comments(_inline(SHADERS / fname, {fname}))
    items = _items(src)
    funcs = {}
    order = []
    for it in items:
        if it[0] == "func":
            name = _func_name(it[1])
            funcs.setdefault(name, []).append(it)
            if name not in order:
                order.append(name)
    # functions reachable from the entry
    need, todo = set(), [entry]
    while todo:
        f = todo.pop()
        if f in need or f not in funcs:
            continue
        need.add(f)
        for it in funcs[f]:
            for ident in set(re.findall(r"\b(\w+)\s*\(", it[2])):
                if ident in funcs and ident not in need:
                    todo.append(ident)
    payloads: dict = {}
    inpayload: list = []
    out = [f"namespace {stage} {{", "using namespace glsl;", USING, "typedef dvec2 vec2; typedef dvec3 vec3; typedef dvec4 vec4;"]
    for it in items:
        if it[0] == "pp":
            if it[1].startswith("#define"):
                out.append(it[1])
        elif it[0] == "decl":
            d = _decl(it[1], stage, payloads, inpayload)
            if d:
                out.append(d)
    for name in order:
        if name not in need:
            continue
        for it in funcs[name]:
            head = _params(it[1])
            body = it[2]
            if name == "main":
                head = "void stage_main()"
            out.append(head + " " + body)
    text = "\n".join(out)
    for p in inpayload:  # the incoming payload is read through the pointer the harness sets
        text = re.sub(rf"\b{p}\b(?!__in)", f"(*{p}__in)", text)
        text = text.replace(f"(*{p}__in)__in", f"{p}__in")
    # traceRayEXT(..., location) -> the stage's payload variable for that location
    if payloads:
        cases = " ".join(f"if (loc == {k}) return &{v};" for k, v in sorted(payloads.items()))
        text = text.replace("using namespace glsl;", "using namespace glsl;\nvoid* payloadAt(int loc);", 1)
        text += f"\nvoid* payloadAt(int loc) {{ {cases} return nullptr; }}"
        text = re.sub(r"\btraceRayEXT\s*\(", f"traceRay_{pipeline}(payloadAt, ", text)
    return text + f"\n}}  // namespace {stage}\n"


def generate() -> Path:
    GEN.mkdir(parents=True, exist_ok=True)
    parts = ["// Generated by oracle/ref_shader/build_ref.py from the reference's shader sources. Do not commit.",
             "#define float double"]
    for stage, (fname, pipeline, entry) in STAGES.items():
        parts.append(translate_stage(stage, fname, pipeline, entry))
    parts.append("#undef float")
    out = GEN / "stages.inc"
    out.write_text("\n".join(parts))
    return out


def build_if_available(force: bool = False) -> Path | None:
    """Builds oracle/_ref/libddgi_refshader.so when the reference sources are present; returns its path
    or None."""
    if not (SHADERS / STAGES["rgen"][0]).is_file():
        return None
    deps = [HERE / "build_ref.py", HERE / "glsl_shim.hpp", HERE / "ref_harness.cpp", ORACLE / "ddgi_oracle.cpp"]
    if LIB.exists() and not force and all(p.stat().st_mtime <= LIB.stat().st_mtime for p in deps):
        return LIB
    generate()
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-pthread", f"-I{GEN}", f"-I{HERE}",
           str(HERE / "ref_harness.cpp"), str(ORACLE / "ddgi_oracle.cpp"), "-o", str(LIB)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference shader build failed:\n" + r.stderr[-6000:])
    return LIB


if __name__ == "__main__":
    print(build_if_available(force="--force" in sys.argv))
