"""Translates a reference GLSL compute shader into C++ that compiles against
oracle/glsl_prelude.hpp (TEST INFRASTRUCTURE: run by oracle/Makefile's `ref`
target; its output goes to oracle/_ref/ only and is never committed).

usage: glsl_cpp.py SHADER.cs OUT.cpp NAMESPACE

The translation is textual and keeps every statement of the shader as it is:
  - comments and `#version` / `#extension` lines are dropped;
  - `layout(local_size_x = N) in;` becomes the workgroup-size constant;
  - a buffer block holding one unsized array becomes a pointer of that type,
    a block with members (and a uniform block) a struct plus one instance;
  - `main` becomes `shader_main`;
  - floating literals get an `f` (GLSL float literals are single precision);
  - arrays returned or declared with initialisers become std::array;
  - each shader's remaining GLSL-only forms (implicit int-to-float vector
    conversions, swizzles of temporaries) are rewritten by the exact
    replacements in FIXUPS, each of which must match.
"""
from __future__ import annotations

import re
import sys
from pathlib import Path

# exact (old, new) replacements per shader, keyed by the path's last two parts
_BATCHED = [
    # GLSL converts ivec2 to vec2 implicitly in mixed arithmetic
    ("uniforms.imageSize.xy * (projCenter.xy", "vec2(uniforms.imageSize) * (projCenter.xy"),
    ("uniforms.imageSize.xy * (projEdge.xy", "vec2(uniforms.imageSize) * (projEdge.xy"),
    ("* 0.5f + 0.5f) * uniforms.imageSize;", "* 0.5f + 0.5f) * vec2(uniforms.imageSize);"),
    # swizzles of temporaries: glm's swizzle members need an lvalue vector
    ("(file.world * vec4(wgMin, 1.0f)).xyz", "vec3(file.world * vec4(wgMin, 1.0f))"),
    ("(file.world * vec4(wgMax, 1.0f)).xyz", "vec3(file.world * vec4(wgMax, 1.0f))"),
]
FIXUPS = {
    "compute_loop_las/render.cs": _BATCHED,
    "compute_loop_las2/render.cs": _BATCHED,
    "compute_loop_las_hqs/depth.cs": _BATCHED[:3],
    "compute_loop_las_hqs/color.cs": _BATCHED,
    "compute_loop_las/resolve.cs": [],
    "compute_loop_las_hqs/resolve.cs": [
        # x / 0 traps in C++; GLSL leaves it undefined, and the shader
        # overwrites r, g, b where count is 0
        ("uint32_t r = R / count;", "uint32_t r = glsl_udiv(R, count);"),
        ("uint32_t g = G / count;", "uint32_t g = glsl_udiv(G, count);"),
        ("uint32_t b = B / count;", "uint32_t b = glsl_udiv(B, count);"),
    ],
    "compute_2021_earlyz/render.cs": [
        ("* 0.5f + 0.5f) * uImageSize;", "* 0.5f + 0.5f) * vec2(uImageSize);"),
    ],
    "compute_2021_earlyz/resolve.cs": [],
    "compute_2021_dedup/render.cs": [
        ("* 0.5f + 0.5f) * uImageSize;", "* 0.5f + 0.5f) * vec2(uImageSize);"),
    ],
    "compute_2021_earlyz_reduce/render.cs": [
        ("* 0.5f + 0.5f) * uImageSize;", "* 0.5f + 0.5f) * vec2(uImageSize);"),
    ],
    "compute_loop_nodes/render.cs": [
        ("uniforms.imageSize.xy * (projCenter.xy", "vec2(uniforms.imageSize) * (projCenter.xy"),
        ("uniforms.imageSize.xy * (projEdge.xy", "vec2(uniforms.imageSize) * (projEdge.xy"),
        ("* 0.5f + 0.5f) * uniforms.imageSize;", "* 0.5f + 0.5f) * vec2(uniforms.imageSize);"),
        # GLSL's min(uint, int) converts the literal; C++ needs it unsigned
        ("loopSize = min(loopSize, 500);", "loopSize = min(loopSize, 500u);"),
    ],
}


def translate(src: str, key: str) -> str:
    # comments out first (the shaders hold no string literals)
    src = re.sub(r"/\*.*?\*/", " ", src, flags=re.S)
    src = re.sub(r"//[^\n]*", "", src)
    lines = [l for l in src.splitlines() if not re.match(r"\s*#\s*(version|extension)\b", l)]
    s = "\n".join(lines) + "\n"
    def wgsize(m):
        y = re.search(r"local_size_y\s*=\s*(\d+)", m.group(0))
        return f"static const uvec3 gl_WorkGroupSize({m.group(1)}u, {y.group(1) if y else 1}u, 1u);"

    s = re.sub(r"layout\s*\(\s*local_size_x\s*=\s*(\d+)[^)]*\)\s*in\s*;", wgsize, s)
    s = re.sub(r"layout\s*\([^)]*\)\s*(?:(?:coherent|readonly|writeonly|restrict)\s+)*uniform\s+uimage2D\s+(\w+)\s*;",
               r"static uimage2D \1;", s)
    s = re.sub(r"layout\s*\([^)]*\)\s*buffer\s+\w+\s*\{\s*(\w+)\s+(\w+)\s*\[\s*\]\s*;\s*\}\s*;",
               r"static \1* \2 = nullptr;", s)

    def block(m):
        name, body, inst = m.group(1), m.group(2), m.group(3)
        body = re.sub(r"(\w+)\s+(\w+)\s*\[\s*\]\s*;", r"\1* \2;", body)
        return f"struct {name} {{{body}}};\nstatic {name} {inst};"

    s = re.sub(r"layout\s*\([^)]*\)\s*(?:buffer|uniform)\s+(\w+)\s*\{(.*?)\}\s*(\w+)\s*;", block, s,
               flags=re.S)
    # a buffer block with one unsized array and no instance name, any layout
    s = re.sub(r"layout\s*\([^)]*\)\s*buffer\s+\w+\s*\{\s*(\w+)\s+(\w+)\s*\[\s*\]\s*;\s*\}\s*;",
               r"static \1* \2 = nullptr;", s)
    s = re.sub(r"layout\s*\([^)]*\)\s*uniform\s+(\w+)\s+(\w+)\s*;", r"static \1 \2;", s)
    s = re.sub(r"(?m)^(\s*)uniform\s+(\w+)\s+(\w+)\s*;", r"\1static \2 \3;", s)
    s = re.sub(r"\bvoid\s+main\s*\(\s*\)", "void shader_main()", s)
    s = re.sub(r"(?<![\w.])(\d+\.\d*(?:[eE][+-]?\d+)?|\.\d+(?:[eE][+-]?\d+)?)(?![\w.])", r"\1f", s)
    s = re.sub(r"\b(\w+)\[(\d+)\]\s+(\w+)\s*\(", r"std::array<\1, \2> \3(", s)
    s = re.sub(r"\b(\w+)\s+(\w+)\s*\[(\d+)\]\s*=\s*\{", r"std::array<\1, \3> \2 = {", s)
    s = re.sub(r"\b(\w+)\[\]\s+(\w+)\s*=", r"auto \2 =", s)
    for old, new in FIXUPS.get(key, []):
        if old not in s:
            raise SystemExit(f"glsl_cpp: fix-up not found in {key}: {old!r}")
        s = s.replace(old, new)
    return s


def main() -> None:
    shader, out, ns = Path(sys.argv[1]), Path(sys.argv[2]), sys.argv[3]
    key = "/".join(shader.parts[-2:])
    body = translate(shader.read_text(), key)
    out.write_text(f"// translated by oracle/glsl_cpp.py from {key}; not committed\n"
                   f'#include "glsl_prelude.hpp"\nnamespace {ns} {{\n{body}}}  // namespace {ns}\n')


if __name__ == "__main__":
    main()
