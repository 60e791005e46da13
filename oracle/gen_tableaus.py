#!/usr/bin/env python3
"""Test infrastructure: emit ``oracle_tableaus.h`` for the CPU oracle.

The oracle is a CPU restatement of the reference used only to check the CUDA
path.  Its coefficients are read straight from the reference's Julia tableau
files (independently of the product's own generator) and laid out as dense,
1-based explicit Runge-Kutta tables with a presence mask, so the oracle can sum
exactly the terms the reference sums, in the reference's order:

* Tsit5  lib/OrdinaryDiffEqTsit5/src/tsit_tableaus.jl:45-101,244-276
* Vern7  lib/OrdinaryDiffEqVerner/src/verner_tableaus.jl:648-716,880-972,1129-1205
* Vern9  lib/OrdinaryDiffEqVerner/src/verner_tableaus.jl:3608-3743
* Rodas5P lib/OrdinaryDiffEqRosenbrock/src/rosenbrock_tableaus.jl:23-72

usage: python gen_tableaus.py <reference-root> [out.h]
"""
import os
import re
import sys

LIT = r"(-?[0-9][0-9_]*(?:\.[0-9]*)?(?:[eE][-+]?[0-9]+)?)"
CF = r"where \{\s*T <: CompiledFloats,\s*T2 <: CompiledFloats,?\s*\}"


def block(text, head):
    m = re.search(head, text)
    if not m:
        raise SystemExit("missing " + head)
    return text[m.end(): text.index("\nend", m.end())]


def values(body):
    d = {}
    for line in body.splitlines():
        line = line.split("#", 1)[0].strip()
        m = re.match(r"^(\w+)\s*=\s*convert\(\s*T2?\s*,\s*" + LIT + r"\s*\)$", line)
        if m:
            d[m.group(1)] = m.group(2).replace("_", "")
    return d


def dbl(s):
    s = str(s)
    return s + ".0" if re.fullmatch(r"-?[0-9]+", s) else s


class Table:
    def __init__(self, s):
        self.s = s
        self.A = [[None] * (s + 1) for _ in range(s + 1)]
        self.c = [None] * (s + 1)
        self.b = [None] * (s + 1)
        self.bt = [None] * (s + 1)

    def emit(self, name):
        s = self.s
        out = ["// %s: %d stages, 1-based; *_m = 1 where the reference has the term" % (name, s)]

        def arr1(tag, v):
            out.append("static const double %s_%s[%d] = {%s};" % (name, tag, s + 1, ", ".join(dbl(x or 0) for x in v)))
            out.append("static const unsigned char %s_%s_m[%d] = {%s};" % (name, tag, s + 1, ", ".join("1" if x is not None else "0" for x in v)))

        out.append("static const double %s_A[%d][%d] = {%s};" % (name, s + 1, s + 1, ", ".join("{" + ", ".join(dbl(x or 0) for x in r) + "}" for r in self.A)))
        out.append("static const unsigned char %s_A_m[%d][%d] = {%s};" % (name, s + 1, s + 1, ", ".join("{" + ", ".join("1" if x is not None else "0" for x in r) + "}" for r in self.A)))
        arr1("c", self.c)
        arr1("b", self.b)
        arr1("bt", self.bt)
        return out


def main():
    ref = sys.argv[1]
    out = sys.argv[2] if len(sys.argv) > 2 else os.path.join(os.path.dirname(os.path.abspath(__file__)), "oracle_tableaus.h")
    tsit = open(os.path.join(ref, "lib/OrdinaryDiffEqTsit5/src/tsit_tableaus.jl")).read()
    vern = open(os.path.join(ref, "lib/OrdinaryDiffEqVerner/src/verner_tableaus.jl")).read()
    ros = open(os.path.join(ref, "lib/OrdinaryDiffEqRosenbrock/src/rosenbrock_tableaus.jl")).read()
    lines = ["// Test infrastructure (oracle only). Generated by oracle/gen_tableaus.py; do not edit.", "#pragma once"]

    # Tsit5: stage i (2..7) at t + c_{i-1} dt; row 7 is the solution (FSAL).
    v = values(block(tsit, r"@fold function Tsit5ConstantCacheActual\(\s*::Type\{T\},\s*::Type\{T2\}\s*\)\s*" + CF))
    t = Table(7)
    for k, x in v.items():
        m = re.fullmatch(r"a(\d)(\d)", k)
        if m:
            t.A[int(m.group(1))][int(m.group(2))] = x
        m = re.fullmatch(r"c(\d)", k)
        if m:
            t.c[int(m.group(1)) + 1] = x
        m = re.fullmatch(r"btilde(\d)", k)
        if m:
            t.bt[int(m.group(1))] = x
    t.c[1] = "0"
    for j in range(1, 7):
        t.b[j] = t.A[7][j]
    lines += t.emit("TSIT5")
    r = values(block(tsit, r"@fold function Tsit5Interp\(::Type\{T\}\) where \{T <: CompiledFloats\}"))
    # r[i][p]: b_i(theta) = sum_p r_ip theta^p
    R = [[r.get("r%d%d" % (i, p), "0") for p in range(0, 5)] for i in range(0, 8)]
    lines.append("static const double TSIT5_R[8][5] = {%s};" % ", ".join("{" + ", ".join(dbl(x) for x in row) + "}" for row in R))

    # Vern7: stage i (2..8) at c_i, stages 9 and 10 at t + dt.
    v = values(block(vern, r"@fold function Vern7Tableau\(\s*::Type\{T\},\s*::Type\{T2\}\s*\)\s*" + CF))
    t = Table(16)
    for k, x in v.items():
        m = re.fullmatch(r"a(\d\d)(\d)", k)
        if m:
            t.A[int(m.group(1))][int(m.group(2))] = x
        m = re.fullmatch(r"c(\d+)", k)
        if m:
            t.c[int(m.group(1))] = x
        m = re.fullmatch(r"b(\d+)", k)
        if m:
            t.b[int(m.group(1))] = x
        m = re.fullmatch(r"btilde(\d+)", k)
        if m:
            t.bt[int(m.group(1))] = x
    t.c[1] = "0"
    t.c[9] = "1"
    t.c[10] = "1"
    x = values(block(vern, r"@fold function Vern7ExtraStages\(\s*::Type\{T\},\s*::Type\{T2\}\s*\)\s*" + CF))
    for k, val in x.items():
        m = re.fullmatch(r"a(\d\d)(\d\d)", k)
        if m:
            t.A[int(m.group(1))][int(m.group(2))] = val
        m = re.fullmatch(r"c(\d+)", k)
        if m:
            t.c[int(m.group(1))] = val
    lines += t.emit("VERN7")
    r = values(block(vern, r"@fold function Vern7InterpolationCoefficients\(::Type\{T\}\) where \{T <: CompiledFloats\}"))
    R = [[r.get("r%02d%d" % (i, p), "0") for p in range(0, 8)] for i in range(0, 17)]
    lines.append("static const double VERN7_R[17][8] = {%s};" % ", ".join("{" + ", ".join(dbl(x) for x in row) + "}" for row in R))

    # Vern9: stage i (2..14) at c_{i-1}; stages 15, 16 at t + dt.
    v = values(block(vern, r"@fold function Vern9Tableau\(\s*::Type\{T\},\s*::Type\{T2\}\s*\)\s*" + CF))
    t = Table(16)
    for k, x in v.items():
        m = re.fullmatch(r"a(\d\d)(\d\d)", k)
        if m:
            t.A[int(m.group(1))][int(m.group(2))] = x
        m = re.fullmatch(r"c(\d+)", k)
        if m:
            t.c[int(m.group(1)) + 1] = x
        m = re.fullmatch(r"b(\d+)", k)
        if m:
            t.b[int(m.group(1))] = x
        m = re.fullmatch(r"btilde(\d+)", k)
        if m:
            t.bt[int(m.group(1))] = x
    t.c[1] = "0"
    t.c[15] = "1"
    t.c[16] = "1"
    lines += t.emit("VERN9")

    # Rodas5P.
    def mat(name):
        body = re.search(r"const " + name + r" = \[(.*?)\n\]", ros, re.S).group(1)
        return [ln.split() for ln in body.strip().splitlines()]

    def vec(name):
        body = re.search(r"const " + name + r" = \[(.*?)\]", ros, re.S).group(1)
        return [x.strip() for x in body.replace("\n", " ").split(",") if x.strip()]

    A, C, H = mat("RODAS5PA"), mat("RODAS5PC"), mat("RODAS5PH")
    gamma = re.search(r"function Rodas5PTableau\(.*?gamma = " + LIT, ros, re.S).group(1)
    lines.append("static const double RODAS5P_GAMMA = %s;" % dbl(gamma))
    lines.append("static const double RODAS5P_A[8][8] = {%s};" % ", ".join("{" + ", ".join(dbl(x) for x in row) + "}" for row in A))
    lines.append("static const double RODAS5P_C[8][7] = {%s};" % ", ".join("{" + ", ".join(dbl(x) for x in row) + "}" for row in C))
    lines.append("static const double RODAS5P_cc[8] = {%s};" % ", ".join(dbl(x) for x in vec("RODAS5Pc")))
    lines.append("static const double RODAS5P_d[8] = {%s};" % ", ".join(dbl(x) for x in vec("RODAS5Pd")))
    lines.append("static const double RODAS5P_H[3][8] = {%s};" % ", ".join("{" + ", ".join(dbl(x) for x in row) + "}" for row in H))
    with open(out, "w") as fh:
        fh.write("\n".join(lines) + "\n")
    print("wrote", out)


if __name__ == "__main__":
    main()
