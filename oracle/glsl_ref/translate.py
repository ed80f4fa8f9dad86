"""ORACLE PIN — test infrastructure only.

Rewrites the reference's GLSL sources into C++ that compiles against
oracle/glsl_ref/glsl.hpp, so the reference's own shader code can be run on
the CPU as a second checker of the oracle.  The rewrite is mechanical and
touches declarations only, never the arithmetic of a function body:

  * drops #version / #extension lines and layout(...) qualifiers
  * float literals get an `f` suffix (GLSL literals are single precision)
  * `inout T x` / `out T x` parameters become references, `in` is dropped
  * uniform/buffer blocks become structs; `T x[]` members become RuntimeArray<T>
  * `T[N] name;` / `T[] name;` resource arrays become Array<T>
  * ray payloads register themselves in the shader's PayloadTable
  * a shader stage is wrapped in `namespace sh_<name>`, its #includes point at
    the rewritten headers, and its #defines are #undef'd at the end

Usage: python translate.py <reference shaders dir> <output dir>
Outputs go to the output directory only (oracle/_ref/gen).
"""
from __future__ import annotations

import re
import sys
from pathlib import Path

FLOAT_LIT = re.compile(r"(?<![\w.])((?:\d+\.\d*|\.\d+)(?:[eE][+-]?\d+)?|\d+[eE][+-]?\d+)(?![\w.])")


def suffix_floats(code: str) -> str:
    out = []
    for line in code.split("\n"):
        if line.lstrip().startswith("#include"):
            out.append(line)
            continue
        # leave comments alone
        cut = line.find("//")
        body, comment = (line, "") if cut < 0 else (line[:cut], line[cut:])
        out.append(FLOAT_LIT.sub(lambda m: m.group(1) + "f", body) + comment)
    return "\n".join(out)


def strip_block_comments(code: str) -> str:
    return re.sub(r"/\*.*?\*/", lambda m: "\n" * m.group(0).count("\n"), code, flags=re.S)


def translate(src: str, stage: str | None) -> str:
    code = strip_block_comments(src)
    code = re.sub(r"^\s*#version.*$", "", code, flags=re.M)
    code = re.sub(r"^\s*#extension.*$", "", code, flags=re.M)
    code = re.sub(r'#include\s+"([\w.]+)"', r'#include "\1.hpp"', code)
    # ray payloads (need the location before layout qualifiers go away)
    code = re.sub(r"layout\s*\(\s*location\s*=\s*(\d+)\s*\)\s*rayPayloadEXT\s+(\w+)\s+(\w+)\s*;",
                  r"\2 \3; static PayloadReg _reg_\3(g_payloads, \1, &\3, sizeof(\3));", code)
    code = re.sub(r"layout\s*\(\s*location\s*=\s*(\d+)\s*\)\s*rayPayloadInEXT\s+(\w+)\s+(\w+)\s*;",
                  r"\2 \3; static PayloadInReg _regin_\3(g_payloads, &\3, sizeof(\3));", code)
    code = re.sub(r"hitAttributeEXT\s+(\w+)\s+(\w+)\s*;", r"\1 \2;", code)
    code = re.sub(r"layout\s*\([^)]*\)\s*in\s*;", "", code)
    code = re.sub(r"layout\s*\([^)]*\)", "", code)
    # interface blocks
    def block(m):
        name, body, inst, arr = m.group(2), m.group(3), m.group(4), m.group(5)
        body = re.sub(r"(\w+)\s+(\w+)\s*\[\s*\]\s*;", r"RuntimeArray<\1> \2;", body)
        decl = f"Array<{name}> {inst};" if arr else f"{name} {inst};"
        return f"struct {name} {{{body}}}; {decl}"
    code = re.sub(r"\b(uniform|buffer)\s+(\w+)\s*\{([^}]*)\}\s*(\w+)\s*(\[\s*\d*\s*\])?\s*;", block, code)
    code = re.sub(r"\b(uniform|readonly|writeonly)\s+", "", code)
    # resource arrays `T[N] name;`
    code = re.sub(r"\b(\w+)\s*\[\s*(\w*)\s*\]\s+(\w+)\s*;", r"Array<\1> \3;", code)
    # stage outputs (`out vec4 fragColor;` at file scope) are plain globals
    code = re.sub(r"^(\s*)out\s+(\w+)\s+(\w+)\s*;", r"\1\2 \3;", code, flags=re.M)
    # parameter qualifiers
    code = re.sub(r"\binout\s+(\w+)\s+(\w+)", r"\1& \2", code)
    code = re.sub(r"\bout\s+(\w+)\s+(\w+)", r"\1& \2", code)
    code = re.sub(r"\bin\s+(\w+)\s*\[\s*(\w+)\s*\]\s+(\w+)", r"const \1 \3[\2]", code)
    code = re.sub(r"\bin\s+(\w+)\s+(\w+)", r"\1 \2", code)
    code = suffix_floats(code)
    defines = re.findall(r"^\s*#define\s+(\w+)", code, flags=re.M)
    if stage:
        head = f"namespace sh_{stage} {{\nusing namespace glsl;\nstatic PayloadTable g_payloads;\n"
        tail = "\n" + "".join(f"#undef {d}\n" for d in defines) + f"}}  // namespace sh_{stage}\n"
        code = head + code + tail
    return "// generated by oracle/glsl_ref/translate.py from the reference's shader source\n" + code


def main(src_dir: str, out_dir: str):
    src, out = Path(src_dir), Path(out_dir)
    out.mkdir(parents=True, exist_ok=True)
    stages = {"shadowRaygen.rgen": "shadowRaygen", "shadow.rmiss": "shadowMiss", "hybridRaygen.rgen": "hybridRaygen",
              "hybridHit.rchit": "hybridHit", "miss.rmiss": "miss", "blur.comp": "blur", "raygen.rgen": "raygen",
              "closesthit.rchit": "closesthit", "postFragment.frag": "post"}
    for name in ("random.glsl", "helpers.glsl", "raycommon.glsl"):
        (out / (name + ".hpp")).write_text(translate((src / name).read_text(), None))
    for name, stage in stages.items():
        (out / (name + ".hpp")).write_text(translate((src / name).read_text(), stage))


if __name__ == "__main__":
    main(sys.argv[1], sys.argv[2])
