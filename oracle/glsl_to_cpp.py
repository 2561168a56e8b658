"""Mechanical GLSL -> C++ transform of the reference's compute shaders (TEST
INFRASTRUCTURE ONLY).

The reference's device code is GLSL 4.50 that needs an OpenGL context, which
this machine does not have.  Its arithmetic is plain scalar and vector code,
so the same source compiles as C++ once a few syntactic differences are
rewritten.  Running the reference's own shader text on the CPU pins the hand
restatement in render_oracle.cpp (and through it the CUDA kernels) to the
reference source rather than to one reader's understanding of it.

Steps, in order (no step looks at what the code means):

1. Assemble the program as the reference's shader loader does
   (src/core/Shader.cpp:180-245): a line that starts with ``@type`` is
   dropped; ``@include f`` inlines shader/f unless f was already included
   (a file is recorded as included after its own text is loaded).
2. Drop comments.
3. Drop ``layout(...)`` qualifiers; mark mutable globals (depth-0 variable
   declarations that are neither ``uniform`` nor ``const``) ``thread_local``,
   because GLSL gives every invocation its own copy; then drop ``uniform``.
4. Parameter qualifiers: ``out T x`` and ``inout T x`` become ``T& x``.
5. Float literals get the ``f`` suffix (GLSL literals are float).
6. Swizzles: ``.r .g .b .a`` become ``.x .y .z .w``; multi-component
   swizzles (``.xy``, ``.rgb`` ...) become calls (``.xy()``, ``.xyz()``).
7. Vector and matrix constructors become braced lists, which C++ evaluates
   left to right as GLSL evaluates arguments (``vec4(sample1D(s), ...)``).
8. ``main`` becomes ``glsl_main``.
9. A ``bind_uniforms(b)`` function is appended that copies every uniform the
   program declares from the member of the same name of `b`, so that the
   driver can set them as the reference's integrator does with
   Shader::set1i / setTexture.

The output is included by oracle/glsl_ref_api.cpp inside ``namespace glsl``
after oracle/glsl_shim.h.
"""
from __future__ import annotations

import re
from pathlib import Path

# name of the generated include -> entry shader
SHADERS = {
    "path_integ_naive": "path_integ_naive.glsl",
    "light_path_integ": "light_path_integ.glsl",
    "triple_path_pass_pt": "triple_path_pass_pt.glsl",
    "triple_path_pass_lpt": "triple_path_pass_lpt.glsl",
}

CTORS = ("vec2", "vec3", "vec4", "ivec2", "mat3")


def assemble(shader_dir: Path, entry: str) -> str:
    """The program text of `entry` with its @include files inlined."""
    out: list[str] = []
    included: set[Path] = set()

    def load(path: Path) -> None:
        for line in path.read_text().splitlines():
            if line.startswith("@"):
                parts = line.split()
                if parts and parts[0] == "@type":
                    continue
                if parts and parts[0] == "@include":
                    inc = shader_dir / parts[1]
                    if inc in included:
                        continue
                    load(inc)
                    included.add(inc)
                    continue
            out.append(line)

    load(shader_dir / entry)
    return "\n".join(out) + "\n"


def strip_comments(src: str) -> str:
    src = re.sub(r"/\*.*?\*/", " ", src, flags=re.S)
    return re.sub(r"//[^\n]*", "", src)


_DECL = re.compile(r"^\s*(?!const\b|uniform\b|struct\b|return\b|#)([A-Za-z_]\w*)\s+([A-Za-z_]\w*)\s*(=[^;]*)?;\s*$")


_UNIFORM = re.compile(r"^\s*(?:layout\s*\([^)]*\)\s*)?uniform\s+\w+\s+(\w+)\s*;", re.M)


def uniform_names(src: str) -> list[str]:
    return _UNIFORM.findall(src)


def mark_globals(src: str) -> str:
    lines = []
    depth = 0
    for line in src.split("\n"):
        line = re.sub(r"\blayout\s*\([^)]*\)\s*", "", line)
        if depth == 0 and _DECL.match(line):
            line = "thread_local " + line.lstrip()
        depth += line.count("{") - line.count("}")
        lines.append(line)
    src = "\n".join(lines)
    return re.sub(r"\buniform\s+", "", src)


def param_qualifiers(src: str) -> str:
    return re.sub(r"\b(?:inout|out)\s+([A-Za-z_]\w*)\s+([A-Za-z_]\w*)", r"\1& \2", src)


_FLOAT = re.compile(r"(?<![\w.])((?:\d+\.\d*|\.\d+)(?:[eE][+-]?\d+)?|\d+[eE][+-]?\d+)(?![\w.])")


def float_literals(src: str) -> str:
    return _FLOAT.sub(lambda m: m.group(1) + "f", src)


_RGBA = str.maketrans("rgba", "xyzw")


def swizzles(src: str) -> str:
    def multi(m):
        return "." + m.group(1).translate(_RGBA) + "()"

    src = re.sub(r"(?<=[\w)\]])\.([xyzw]{2,4}|[rgba]{2,4})\b(?!\s*\()", multi, src)
    return re.sub(r"(?<=[\w)\]])\.([rgba])\b", lambda m: "." + m.group(1).translate(_RGBA), src)


def braced_ctors(src: str) -> str:
    """vecN(...) -> vecN{...} with balanced parentheses."""
    pat = re.compile(r"\b(" + "|".join(CTORS) + r")\s*\(")
    out = []
    i = 0
    while True:
        m = pat.search(src, i)
        if not m:
            out.append(src[i:])
            break
        # a declaration such as `vec3 foo(` is not a constructor call: the name
        # is followed by an identifier there, never by '('
        out.append(src[i:m.start()])
        out.append(m.group(1) + "{")
        j = m.end()
        depth = 1
        k = j
        while depth:
            c = src[k]
            if c == "(":
                depth += 1
            elif c == ")":
                depth -= 1
            k += 1
        out.append(braced_ctors(src[j:k - 1]))
        out.append("}")
        i = k
    return "".join(out)


def transform(src: str) -> str:
    src = strip_comments(src)
    names = uniform_names(src)
    src = mark_globals(src)
    src = param_qualifiers(src)
    src = float_literals(src)
    src = swizzles(src)
    src = braced_ctors(src)
    src = re.sub(r"\bvoid\s+main\s*\(", "void glsl_main(", src)
    body = "".join(f"    {n} = b.{n};\n" for n in names)
    return src + "\ntemplate <class B>\nvoid bind_uniforms(const B& b) {\n" + body + "}\n"


def transform_program(shader_dir: Path, entry: str) -> str:
    head = (f"// Generated by oracle/glsl_to_cpp.py from the reference's src/shader/{entry} and the files\n"
            "// it includes.  TEST INFRASTRUCTURE ONLY; never committed.\n")
    return head + transform(assemble(Path(shader_dir), entry))


if __name__ == "__main__":
    import sys

    d = Path(sys.argv[1]) if len(sys.argv) > 1 else Path("/root/reference/src/shader")
    print(transform_program(d, "path_integ_naive.glsl"))
