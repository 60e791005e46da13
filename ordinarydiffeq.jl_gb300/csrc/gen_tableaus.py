#!/usr/bin/env python3
"""Generate ``tableaus.h`` (method coefficients for the device kernels).

The coefficients are data that must equal the reference's exactly, so they are
read from the reference's Julia sources rather than retyped:

* Tsit5:  lib/OrdinaryDiffEqTsit5/src/tsit_tableaus.jl:45-101 (Float64 branch of
  ``Tsit5ConstantCacheActual``) and :244-276 (``Tsit5Interp``).
* Vern7:  lib/OrdinaryDiffEqVerner/src/verner_tableaus.jl:1129-1205 (``Vern7Tableau``),
  :648-716 (``Vern7ExtraStages``), :880-972 (``Vern7InterpolationCoefficients``).
* Rodas5P: lib/OrdinaryDiffEqRosenbrock/src/rosenbrock_tableaus.jl:23-72
  (``RODAS5PA/C/c/d/H`` and ``Rodas5PTableau``).
* Rosenbrock23: rosenbrock_tableaus.jl:6-10 (``c32 = 6 + sqrt(2)``,
  ``d = 1 / (2 + sqrt(2))``): expressions, evaluated here in IEEE double with
  the same correctly rounded operations Julia's Float64 arithmetic performs.

Each Julia literal is copied verbatim as a C++ double literal, so the C++ parser
rounds it to the same IEEE double as Julia's parser does.  Run once in a
checkout that has the reference tree; the output is committed.

usage: python gen_tableaus.py <reference-root> [out.h]
"""
import os
import re

import numpy as np
import sys

LIT = r"(-?[0-9][0-9_]*(?:\.[0-9]*)?(?:[eE][-+]?[0-9]+)?)"


def fold_block(text, header_regex):
    """Return the body of the first ``@fold function`` whose header matches."""
    m = re.search(header_regex, text)
    if not m:
        raise SystemExit("block not found: " + header_regex)
    start = m.end()
    end = text.index("\nend", start)
    return text[start:end]


def assignments(body):
    out = {}
    for line in body.splitlines():
        line = line.split("#", 1)[0].strip()
        m = re.match(r"^(\w+)\s*=\s*convert\(\s*T2?\s*,\s*" + LIT + r"\s*\)$", line)
        if m:
            out[m.group(1)] = m.group(2).replace("_", "")
    return out


def julia_matrix(text, name):
    m = re.search(r"const " + name + r" = \[(.*?)\n\]", text, re.S)
    if not m:
        raise SystemExit("matrix not found: " + name)
    rows = []
    for line in m.group(1).strip().splitlines():
        vals = line.strip().rstrip(",").replace(",", " ").split()
        rows.append([v for v in vals])
    return rows


def as_double(lit):
    lit = lit.strip()
    if re.fullmatch(r"-?[0-9]+", lit):
        return lit + ".0"
    return lit


def main():
    ref = sys.argv[1]
    out = sys.argv[2] if len(sys.argv) > 2 else os.path.join(os.path.dirname(__file__), "tableaus.h")
    tsit = open(os.path.join(ref, "lib/OrdinaryDiffEqTsit5/src/tsit_tableaus.jl")).read()
    vern = open(os.path.join(ref, "lib/OrdinaryDiffEqVerner/src/verner_tableaus.jl")).read()
    ros = open(os.path.join(ref, "lib/OrdinaryDiffEqRosenbrock/src/rosenbrock_tableaus.jl")).read()

    compiled = r"where \{\s*T <: CompiledFloats,\s*T2 <: CompiledFloats,?\s*\}"
    blocks = [
        ("TSIT5", assignments(fold_block(tsit, r"@fold function Tsit5ConstantCacheActual\(\s*::Type\{T\},\s*::Type\{T2\}\s*\)\s*" + compiled))),
        ("TSIT5I", assignments(fold_block(tsit, r"@fold function Tsit5Interp\(::Type\{T\}\) where \{T <: CompiledFloats\}"))),
        ("VERN7", assignments(fold_block(vern, r"@fold function Vern7Tableau\(\s*::Type\{T\},\s*::Type\{T2\}\s*\)\s*" + compiled))),
        ("VERN7X", assignments(fold_block(vern, r"@fold function Vern7ExtraStages\(\s*::Type\{T\},\s*::Type\{T2\}\s*\)\s*" + compiled))),
        ("VERN7I", assignments(fold_block(vern, r"@fold function Vern7InterpolationCoefficients\(::Type\{T\}\) where \{T <: CompiledFloats\}"))),
    ]
    lines = [
        "// Generated by gen_tableaus.py from the reference's Julia tableau sources; do not edit.",
        "// Tsit5: lib/OrdinaryDiffEqTsit5/src/tsit_tableaus.jl:45-101,244-276",
        "// Vern7: lib/OrdinaryDiffEqVerner/src/verner_tableaus.jl:648-716,880-972,1129-1205",
        "// Rodas5P: lib/OrdinaryDiffEqRosenbrock/src/rosenbrock_tableaus.jl:23-72",
        "// Rosenbrock23: lib/OrdinaryDiffEqRosenbrock/src/rosenbrock_tableaus.jl:6-10",
        "#pragma once",
        "#ifndef __CUDACC_RTC__",
        "#include <cuda_runtime.h>",
        "#endif",
        "namespace odegb {",
        "namespace tab {",
    ]
    for prefix, vals in blocks:
        lines.append("// " + prefix)
        for k, v in vals.items():
            lines.append("constexpr double %s_%s = %s;" % (prefix, k, as_double(v)))
    A = julia_matrix(ros, "RODAS5PA")
    C = julia_matrix(ros, "RODAS5PC")
    H = julia_matrix(ros, "RODAS5PH")
    c = re.search(r"const RODAS5Pc = \[(.*?)\]", ros, re.S).group(1).replace("\n", " ").split(",")
    d = re.search(r"const RODAS5Pd = \[(.*?)\]", ros, re.S).group(1).replace("\n", " ").split(",")
    c = [x.strip() for x in c if x.strip()]
    d = [x.strip() for x in d if x.strip()]
    gamma = re.search(r"function Rodas5PTableau\(.*?gamma = " + LIT, ros, re.S).group(1)
    lines.append("// RODAS5P (8 stages): A lower triangular 8x8, C 8x7, c 8, d 8, H 3x8.")
    lines.append("// Accessors are constexpr functions so device code folds them to immediates.")
    lines.append("constexpr double RODAS5P_GAMMA = %s;" % as_double(gamma))

    def f32_split(lit):
        # x = hi + lo with hi = float(x) (round to nearest) and lo = float(x - hi),
        # both written as exact hexadecimal float literals
        x = float(as_double(lit))
        hi = float(np.float32(x))
        lo = float(np.float32(x - hi))
        return hi.hex() + "f", lo.hex() + "f"

    def accessor(name, rows, two_d=True):
        if two_d:
            body = ", ".join("{" + ", ".join(as_double(v) for v in r) + "}" for r in rows)
            lines.append("__host__ __device__ constexpr double %s(int i, int j) {" % name)
            lines.append("    constexpr double t[%d][%d] = {%s};" % (len(rows), len(rows[0]), body))
            lines.append("    return t[i][j];")
            lines.append("}")
            for part, tag in ((0, "HI"), (1, "LO")):
                body = ", ".join("{" + ", ".join(f32_split(v)[part] for v in r) + "}" for r in rows)
                lines.append("__host__ __device__ constexpr float %s_%s(int i, int j) {" % (name, tag))
                lines.append("    constexpr float t[%d][%d] = {%s};" % (len(rows), len(rows[0]), body))
                lines.append("    return t[i][j];")
                lines.append("}")
        else:
            body = ", ".join(as_double(v) for v in rows)
            lines.append("__host__ __device__ constexpr double %s(int i) {" % name)
            lines.append("    constexpr double t[%d] = {%s};" % (len(rows), body))
            lines.append("    return t[i];")
            lines.append("}")
            for part, tag in ((0, "HI"), (1, "LO")):
                body = ", ".join(f32_split(v)[part] for v in rows)
                lines.append("__host__ __device__ constexpr float %s_%s(int i) {" % (name, tag))
                lines.append("    constexpr float t[%d] = {%s};" % (len(rows), body))
                lines.append("    return t[i];")
                lines.append("}")

    accessor("RODAS5P_A", A)
    accessor("RODAS5P_C", C)
    accessor("RODAS5P_c", c, two_d=False)
    accessor("RODAS5P_d", d, two_d=False)
    accessor("RODAS5P_H", H)

    # Dense 1-based explicit-RK tables (rows = stages, zero where the reference
    # has no term) with presence masks, for the generic stage loops.
    def erk_tables(prefix, vals, extra, S, row_digits, c_of_stage):
        A = [["0.0"] * (S + 1) for _ in range(S + 1)]
        M = [[0] * (S + 1) for _ in range(S + 1)]
        for k, v in list(vals.items()) + list(extra.items()):
            m = re.fullmatch(r"a(\d{%d})(\d+)" % row_digits, k) if row_digits else None
            if k.startswith("a") and len(k) == 5 and prefix == "VERN7":  # a1101 style (extra stages)
                m = re.fullmatch(r"a(\d\d)(\d\d)", k)
            if m:
                i, j = int(m.group(1)), int(m.group(2))
                A[i][j] = as_double(v)
                M[i][j] = 1
        cvec = ["0.0"] * (S + 1)
        for i in range(2, S + 1):
            cvec[i] = as_double(c_of_stage(i))
        accessor(prefix + "_A", A)
        lines.append("__host__ __device__ constexpr bool %s_AM(int i, int j) {" % prefix)
        lines.append("    constexpr bool t[%d][%d] = {%s};" % (S + 1, S + 1, ", ".join("{" + ", ".join("true" if x else "false" for x in r) + "}" for r in M)))
        lines.append("    return t[i][j];")
        lines.append("}")
        accessor(prefix + "_CS", cvec, two_d=False)

    tv = dict(blocks[0][1])
    # Tsit5: a<i><j> single digits, stage i at c_{i-1}; row 7 is the solution (FSAL)
    erk_tables("TSIT5", tv, {}, 7, 1, lambda i: tv["c%d" % (i - 1)] if i <= 7 else "1")
    bt = ["0.0"] * 8
    for j in range(1, 8):
        bt[j] = as_double(tv["btilde%d" % j])
    accessor("TSIT5_BT", bt, two_d=False)
    ti = dict(blocks[1][1])
    R = [[as_double(ti.get("r%d%d" % (i, q), "0")) for q in range(5)] for i in range(8)]
    accessor("TSIT5_R", R)
    vv = dict(blocks[2][1])
    vx = dict(blocks[3][1])
    def vern_c(i):
        if i <= 8:
            return vv["c%d" % i]
        if i <= 10:
            return "1"
        return vx["c%d" % i]
    erk_tables("VERN7", vv, vx, 16, 2, vern_c)
    b = ["0.0"] * 17
    bm = [0] * 17
    btl = ["0.0"] * 17
    btm = [0] * 17
    for k, v in vv.items():
        m = re.fullmatch(r"b(\d+)", k)
        if m:
            b[int(m.group(1))] = as_double(v)
            bm[int(m.group(1))] = 1
        m = re.fullmatch(r"btilde(\d+)", k)
        if m:
            btl[int(m.group(1))] = as_double(v)
            btm[int(m.group(1))] = 1
    accessor("VERN7_B", b, two_d=False)
    accessor("VERN7_BT", btl, two_d=False)
    for name, mask in (("VERN7_BM", bm), ("VERN7_BTM", btm)):
        lines.append("__host__ __device__ constexpr bool %s(int j) {" % name)
        lines.append("    constexpr bool t[17] = {%s};" % ", ".join("true" if x else "false" for x in mask))
        lines.append("    return t[j];")
        lines.append("}")
    vi = dict(blocks[4][1])
    R7 = [[as_double(vi.get("r%02d%d" % (i, q), "0")) for q in range(8)] for i in range(17)]
    accessor("VERN7_R", R7)

    # Rosenbrock23: the two expressions of Rosenbrock23Tableau, checked against the source
    body = fold_block(ros, r"function Rosenbrock23Tableau\(::Type\{T\}\) where \{T\}")
    if "convert(T, 6 + sqrt(2))" not in body or "convert(T, 1 / (2 + sqrt(2)))" not in body:
        raise SystemExit("Rosenbrock23Tableau changed: " + body)
    import math
    c32 = 6.0 + math.sqrt(2.0)
    dd = 1.0 / (2.0 + math.sqrt(2.0))
    lines.append("// ROSENBROCK23: c32 = 6 + sqrt(2), d = 1 / (2 + sqrt(2)) in Float64")
    for name, x in (("ROS23_C32", c32), ("ROS23_D", dd)):
        hi = float(np.float32(x))
        lo = float(np.float32(x - hi))
        lines.append("constexpr double %s = %s;  // %r" % (name, x.hex(), x))
        lines.append("constexpr float %s_HI = %sf;" % (name, hi.hex()))
        lines.append("constexpr float %s_LO = %sf;" % (name, lo.hex()))
    lines.append("}  // namespace tab")
    lines.append("}  // namespace odegb")
    with open(out, "w") as fh:
        fh.write("\n".join(lines) + "\n")
    print("wrote", out, sum(len(v) for _, v in blocks), "named coefficients")


if __name__ == "__main__":
    main()
