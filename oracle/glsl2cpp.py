"""Test infrastructure (oracle) — NOT part of the product.

Rewrites the reference's compute shader (ray-trace-compute.comp and the two
files it includes) into C++ that compiles against oracle/shim/glsl.h, so the
shader's own source can run on the host as a checker. Only mechanical,
meaning-preserving rewrites are applied; the output goes to oracle/_ref/ and
is never committed:

  * `#include "include/x.glsl"` is inlined (recursively rewritten);
  * `#version` and the `layout(local_size...) in;` line are dropped;
  * the uniform block becomes a struct plus an extern instance, image
    uniforms extern image2D objects, and std430 buffer blocks
    `T[] name` extern GlslArray<T> objects (bound by the harness);
  * `in T x` parameters lose the qualifier; `out`/`inout T x` become `T& x`
    (the shader never passes one variable to two such parameters, so
    references behave as GLSL's copy-in/copy-out);
  * fp literals without a suffix get `f` (GLSL literals are float);
  * swizzles (.xyz .zxy .xy .rgb .rgba) become member calls;
  * top-level globals initialised from per-invocation values (rngState)
    become thread_local variables set by glsl_init_globals();
  * local scalars declared without an initialiser get `{}` (GLSL leaves
    them undefined; where the shader reads one, the value never reaches
    its output);
  * vector constructors `vecN(a, b, c)` become `vecN{a, b, c}`: GLSL
    evaluates call arguments left to right (GLSL 4.50, 6.1.1), C++ leaves
    the order of function arguments unspecified but fixes it for braced
    initialisers (random_in_unit_sphere calls random() three times inside
    one constructor);
  * main() becomes glsl_main(); random() becomes glsl_random() (POSIX has a
    random()); imageSize() becomes glsl_imageSize() (main declares a local
    of that name, which GLSL scopes after its initialiser and C++ before).

Usage: python glsl2cpp.py <path to ray-trace-compute.comp> > out.cpp
"""
import os
import re
import sys


def read_inlined(path: str) -> str:
    base = os.path.dirname(path)
    out = []
    for line in open(path, encoding="utf-8").read().splitlines():
        m = re.match(r'\s*#include\s+"([^"]+)"', line)
        if m:
            out.append(read_inlined(os.path.join(base, m.group(1))))
        else:
            out.append(line)
    return "\n".join(out)


def strip_comments(src: str) -> str:
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return re.sub(r"//[^\n]*", "", src)


def braced_constructors(src: str) -> str:
    """vec2/vec3/vec4/ivec2 ( ... ) -> { ... }, with nested parentheses."""
    out, i = [], 0
    pat = re.compile(r"\b(?:vec[234]|ivec2)\s*\(")
    while True:
        m = pat.search(src, i)
        if not m:
            out.append(src[i:])
            return "".join(out)
        out.append(src[i:m.end() - 1] + "{")
        depth, j = 1, m.end()
        while depth:
            c = src[j]
            depth += (c == "(") - (c == ")")
            j += 1
        inner = braced_constructors(src[m.end():j - 1])
        out.append(inner + "}")
        i = j


def translate(src: str) -> str:
    src = strip_comments(src)
    src = re.sub(r"^\s*#version[^\n]*\n", "", src, flags=re.M)
    src = re.sub(r"layout\s*\(\s*local_size[^)]*\)\s*in\s*;", "", src)
    # Uniform block -> struct + extern instance.
    src = re.sub(r"layout\s*\([^)]*\)\s*uniform\s+(\w+)\s*\{(.*?)\}\s*(\w+)\s*;",
                 lambda m: "struct %s {%s};\nextern %s %s;" % (m.group(1), m.group(2), m.group(1), m.group(3)),
                 src, flags=re.S)
    # Image uniforms.
    src = re.sub(r"layout\s*\([^)]*\)\s*uniform\s+image2D\s+(\w+)\s*;", r"extern image2D \1;", src)
    # std430 buffer blocks holding one runtime-sized array.
    src = re.sub(r"layout\s*\([^)]*\)\s*(?:readonly\s+)?buffer\s+\w+\s*\{\s*(\w+)\s*\[\s*\]\s*(\w+)\s*;\s*\}\s*;",
                 r"extern GlslArray<\1> \2;", src, flags=re.S)
    # Parameter qualifiers.
    src = re.sub(r"\b(?:inout|out)\s+(\w+)\s+(\w+)", r"\1& \2", src)
    src = re.sub(r"([(,]\s*)in\s+(\w+\s+\w+)", r"\1\2", src)
    # Float literals.
    src = re.sub(r"(?<![\w.])((?:\d+\.\d*|\.\d+)(?:[eE][+-]?\d+)?)(?![fF\w.])", r"\1f", src)
    # Swizzles.
    src = re.sub(r"\.(xyz|zxy|xy|rgba|rgb)\b(?!\s*\()", r".\1()", src)
    src = braced_constructors(src)
    # Renames.
    src = re.sub(r"\brandom\b(?=\s*\()", "glsl_random", src)
    src = re.sub(r"\bimageSize\b(?=\s*\()", "glsl_imageSize", src)
    src = re.sub(r"\bvoid\s+main\s*\(", "void glsl_main(", src)
    # Top-level globals initialised per invocation, and undefined locals.
    out, inits, depth = [], [], 0
    for line in src.split("\n"):
        stripped = line.strip()
        m = re.match(r"^(uint|int|float)\s+(\w+)\s*=\s*(.+);$", stripped)
        if depth == 0 and m and not stripped.startswith("const"):
            out.append("thread_local %s %s;" % (m.group(1), m.group(2)))
            inits.append("  %s = %s;" % (m.group(2), m.group(3)))
        else:
            if depth > 0:
                line = re.sub(r"^(\s*)(float|int|uint|bool)\s+(\w+)\s*;\s*$", r"\1\2 \3{};", line)
            out.append(line)
        depth += line.count("{") - line.count("}")
    out.append("void glsl_init_globals() {\n%s\n}" % "\n".join(inits))
    return '#include "glsl.h"\n' + "\n".join(out) + "\n"


if __name__ == "__main__":
    sys.stdout.write(translate(read_inlined(sys.argv[1])))
