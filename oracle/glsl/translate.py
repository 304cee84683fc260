#!/usr/bin/env python3
"""TEST INFRASTRUCTURE ONLY — turns one of the reference's GLSL compute programs into a C++
translation unit for the host GLSL environment (oracle/glsl/glsl.hpp).

    python translate.py SHADER_DIR PROGRAM OUT.cpp

The shader sources are read where they lie (water/shaders/compute of the reference checkout) and
the output goes to oracle/_ref/ (git-ignored): no reference source is kept in this repository.
The translation rewrites only what C++ spells differently, so that the shader's own statements
run unchanged:

- `#include "x"` is expanded and `#[...]` / `#version` lines dropped, as the reference's
  water/compute_source.gd:expand does before compiling;
- comments are removed;
- storage buffers become pointers (a block with one non-array member becomes a value), images
  become glsl::Image3D, the push-constant block becomes a struct instance, `shared` arrays become
  globals of the translation unit (one workgroup runs at a time), `layout(local_size_x...) in;`
  is dropped;
- `out`/`inout` parameters become references, `precise` is dropped;
- floating-point literals get the `f` suffix (GLSL literals are float);
- multi-component swizzles become calls: `v.xyz` reads a vector value, `v.xyz_w()` is the target
  of an assignment;
- `main` becomes `glsl_main`, and a binding table is generated.

The wall-variant program (COUPLED without COASTAL) has no program file in the reference; it is
coastal.glsl's include list without the offshore-forcing files and with main's coastal branch
left out.
"""
import os
import re
import sys

SHADERS_INCLUDED_BY_COASTAL = ["periodic_index.glslinc", "pressure_core.glslinc", "plic_math.glslinc",
                               "coastal_target.glslinc", "pressure_geometry.glslinc", "height_normal.glslinc",
                               "pressure_iterations.glslinc", "pressure_pass.glslinc", "coupled_motion.glslinc",
                               "coastal_pass.glslinc"]

PROGRAMS = {
    "coastal": {"file": "coastal.glsl"},
    "mg_vectors": {"file": "pressure_mg_cache_vectors.glsl"},
    "mg_build": {"file": "pressure_mg_cache_build.glsl"},
    "mg_coarse": {"file": "pressure_mg_cache_coarse.glsl"},
    "mg_arguments": {"file": "pressure_mg_cache_arguments.glsl"},
    "hierarchy": {"file": "pressure_hierarchy_state.glsl"},
    "coupled": {"text": "#define COUPLED\n"
                        + "".join(f'#include "{f}"\n' for f in SHADERS_INCLUDED_BY_COASTAL
                                  if f not in ("coastal_target.glslinc", "coastal_pass.glslinc"))
                        + "void main(){int op=int(pc.dims_op.w);if(op>=20)motion_pass();else pressure_pass();}\n"},
}


def expand(path, stack=()):
    """water/compute_source.gd:expand: inline includes, drop '#[' lines."""
    if path in stack:
        raise SystemExit(f"cyclic include {path}")
    out = []
    with open(path) as f:
        for line in f.read().split("\n"):
            s = line.strip()
            if s.startswith("#["):
                continue
            if s.startswith("#include"):
                rel = line.split('"')[1]
                out.append(expand(os.path.join(os.path.dirname(path), rel), stack + (path,)))
            else:
                out.append(line)
    return "\n".join(out) + "\n"


def expand_text(text, base):
    out = []
    for line in text.split("\n"):
        if line.strip().startswith("#include"):
            out.append(expand(os.path.join(base, line.split('"')[1])))
        else:
            out.append(line)
    return "\n".join(out)


def preprocess(src):
    """Resolves the conditionals the shaders use (#define X, #ifdef, #ifndef, #elif defined(X),
    #else, #endif), so that the binding table sees only the blocks compiled in."""
    defined, out, stack = set(), [], []  # stack of [active, taken, parent_active]
    for line in src.split("\n"):
        s = line.strip()
        active = all(frame[0] for frame in stack)
        m = re.match(r"#\s*(define|ifdef|ifndef|elif|else|endif)\b\s*(.*)", s)
        if not m:
            if active:
                out.append(line)
            continue
        kind, arg = m.group(1), m.group(2).strip()
        if kind == "define":
            if active:
                defined.add(arg.split()[0])
        elif kind in ("ifdef", "ifndef"):
            cond = (arg in defined) == (kind == "ifdef")
            stack.append([cond, cond])
        elif kind == "elif":
            mm = re.match(r"defined\s*\(?\s*(\w+)\s*\)?$", arg)
            if not mm:
                raise SystemExit(f"unsupported #elif {arg}")
            frame = stack[-1]
            cond = not frame[1] and mm.group(1) in defined
            frame[0] = cond
            frame[1] = frame[1] or cond
        elif kind == "else":
            frame = stack[-1]
            frame[0] = not frame[1]
            frame[1] = True
        else:
            stack.pop()
    return "\n".join(out)


def strip_comments(src):
    src = re.sub(r"/\*.*?\*/", " ", src, flags=re.S)
    return re.sub(r"//[^\n]*", "", src)


TYPES = r"(?:u?vec[234]|ivec[234]|bvec[234]|float|int|uint|bool)"


def translate(src):
    src = strip_comments(src)
    src = re.sub(r"^\s*#version[^\n]*", "", src, flags=re.M)
    src = preprocess(src)
    src = re.sub(r"layout\s*\(\s*local_size_x[^)]*\)\s*in\s*;", "", src)
    bindings = []  # (binding, kind, name, type)

    def buffer_block(m):
        binding = int(re.search(r"binding\s*=\s*(\d+)", m.group(1)).group(1))
        body = m.group(3).strip().rstrip(";")
        mm = re.match(r"(\w+)\s+(\w+)\s*(\[\s*\])?$", body)
        if not mm:
            raise SystemExit(f"unsupported buffer block: {m.group(0)}")
        typ, name, arr = mm.group(1), mm.group(2), mm.group(3)
        bindings.append((binding, "array" if arr else "value", name, typ))
        return f"{typ}* {name} = nullptr;" if arr else f"{typ} {name};"

    src = re.sub(r"layout\s*\(([^)]*)\)\s*(?:(?:readonly|writeonly|coherent|restrict|volatile)\s+)*buffer\s+(\w+)\s*\{([^}]*)\}\s*;",
                 buffer_block, src)

    def image(m):
        binding = int(re.search(r"binding\s*=\s*(\d+)", m.group(1)).group(1))
        bindings.append((binding, "image", m.group(2), "image3D"))
        return f"Image3D {m.group(2)};"

    src = re.sub(r"layout\s*\(([^)]*)\)\s*uniform\s+(?:(?:readonly|writeonly)\s+)*image3D\s+(\w+)\s*;", image, src)
    src = re.sub(r"layout\s*\(\s*push_constant[^)]*\)\s*uniform\s+(\w+)\s*\{", r"struct \1 {", src)
    src = re.sub(r"\bshared\s+(?=" + TYPES + r"\b)", "", src)
    src = re.sub(r"\bprecise\s+", "", src)
    # out / inout parameters (arrays first), then plain `in`
    src = re.sub(r"\b(?:inout|out)\s+(\w+)\s+(\w+)\s*\[\s*(\d+)\s*\]", r"\1 (&\2)[\3]", src)
    src = re.sub(r"\b(?:inout|out)\s+(\w+)\s+(\w+)", r"\1& \2", src)
    src = re.sub(r"([(,]\s*)in\s+(" + TYPES + r")\b", r"\1\2", src)
    # float literals
    src = re.sub(r"(?<![\w.])(\d+\.\d*(?:[eE][+-]?\d+)?|\.\d+(?:[eE][+-]?\d+)?|\d+[eE][+-]?\d+)(?![\w.])", r"\1f", src)
    # swizzles: assignment targets, then reads
    sw = r"(xyzw|xyz|yzw|xy|yz|xz|zw|yx)"
    src = re.sub(r"\." + sw + r"\b(?=\s*(?:[-+*/]?=)(?!=))", r".\1_w()", src)
    src = re.sub(r"\." + sw + r"\b(?!_w\(|\()", r".\1()", src)
    src = re.sub(r"\bvoid\s+main\s*\(", "void glsl_main(", src)
    return src, bindings


def emit(program, src, bindings):
    ns = "ref_" + program
    lines = ['#include "glsl.hpp"', f"namespace {ns} {{", "using namespace glsl;", src, ""]
    lines.append("void bind(int binding, void* ptr) {")
    lines.append("  switch (binding) {")
    for b, kind, name, typ in bindings:
        if kind == "array":
            lines.append(f"    case {b}: {name} = static_cast<{typ}*>(ptr); break;")
        elif kind == "value":
            lines.append(f"    case {b}: {name} = *static_cast<{typ}*>(ptr); break;")
        else:
            lines.append(f"    case {b}: {name} = *static_cast<Image3D*>(ptr); break;")
    lines.append("    default: break;")
    lines.append("  }")
    lines.append("}")
    lines.append("void* push_constants() { return &pc; }")
    lines.append("unsigned push_constant_bytes() { return sizeof(pc); }")
    lines.append("void run(unsigned gx, unsigned gy) { dispatch(glsl_main, uvec3(gx, gy, 1u)); }")
    lines.append(f"}}  // namespace {ns}")
    return "\n".join(lines) + "\n"


def main():
    shader_dir, program, out = sys.argv[1], sys.argv[2], sys.argv[3]
    spec = PROGRAMS[program]
    if "file" in spec:
        src = expand(os.path.join(shader_dir, spec["file"]))
    else:
        src = expand_text(spec["text"], shader_dir)
    code, bindings = translate(src)
    os.makedirs(os.path.dirname(os.path.abspath(out)), exist_ok=True)
    with open(out, "w") as f:
        f.write(emit(program, code, bindings))


if __name__ == "__main__":
    main()
