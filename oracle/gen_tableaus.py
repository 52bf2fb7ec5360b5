#!/usr/bin/env python3
"""Generate the Butcher/Rosenbrock tableau headers from DiffEqGPU.jl's tableau files.

Test-infrastructure / build-time recipe.  It reads the reference's tableau sources
(read-only) and writes two headers with the SAME numbers:

  * ``oracle/tableaus_gen.h``                         -- FP64 literals for the CPU oracle
  * ``diffeqgpu.jl_gb300/csrc/device/tableaus_gen.cuh`` -- FP32 ``__constant__`` arrays for
    the kernels.

The reference writes every coefficient as ``name = convert(T, <Float64 literal>)`` (or
its negation ``-convert(T, ...)``)
(``src/ensemblegpukernel/tableaus/verner_tableaus.jl`` and ``rodas_tableaus.jl``) and
Julia's ``convert(Float32, x::Float64)`` rounds to nearest.  The device header stores
``float(np.float32(np.float64(literal)))`` printed with enough digits to round-trip,
so the kernels see bit-identical coefficients.

Run once in a checkout that has the reference mounted:
    python oracle/gen_tableaus.py /root/reference
The outputs are committed; nothing at run time reads the reference.
"""
import re
import sys
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent.parent

# (table name, file, julia function, first line, last line) -- line ranges are cited in the headers
TABLES = [
    ("vern7", "src/ensemblegpukernel/tableaus/verner_tableaus.jl", "Vern7Tableau"),
    ("vern7x", "src/ensemblegpukernel/tableaus/verner_tableaus.jl", "Vern7ExtraStages"),
    ("vern7i", "src/ensemblegpukernel/tableaus/verner_tableaus.jl", "Vern7InterpolationCoefficients"),
    ("vern9", "src/ensemblegpukernel/tableaus/verner_tableaus.jl", "Vern9Tableau"),
    ("vern9x", "src/ensemblegpukernel/tableaus/verner_tableaus.jl", "Vern9ExtraStages"),
    ("vern9i", "src/ensemblegpukernel/tableaus/verner_tableaus.jl", "Vern9InterpolationCoefficients"),
    ("rodas5p", "src/ensemblegpukernel/tableaus/rodas_tableaus.jl", "Rodas5PTableau"),
    ("rodas4", "src/ensemblegpukernel/tableaus/rodas_tableaus.jl", "Rodas4Tableau"),
    ("kvaerno3", "src/ensemblegpukernel/tableaus/kvaerno_tableaus.jl", "Kvaerno3Tableau"),
    ("kvaerno5", "src/ensemblegpukernel/tableaus/kvaerno_tableaus.jl", "Kvaerno5Tableau"),
]


def derived(tab: str, entries):
    """Coefficients the reference computes from others instead of writing them as literals
    (kvaerno_tableaus.jl:33-38 and :159), evaluated in Float32 like the Float32 tableau:
    Kvaerno3 btilde4 = -γ and its Hermite predictor weights α31, α32 with c2 = 2γ,
    θ = c3/c2; Kvaerno5 btilde7 = -γ."""
    f = np.float32
    d = dict(entries)
    if tab == "kvaerno3":
        g, c3 = f(d["gamma"]), f(d["c3"])
        c2 = f(2) * g
        th = c3 / c2
        th2 = th * th
        w = (f(6) * th * (f(1) - th)) / c2 * g
        a31 = (f(1) + (f(-4) * th + f(3) * th2)) + w
        a32 = (f(-2) * th + f(3) * th2) + w
        return [("btilde4", float(-g)), ("alpha31", float(a31)), ("alpha32", float(a32))]
    if tab == "kvaerno5":
        return [("btilde7", float(-f(d["gamma"])))]
    return []

ASSIGN = re.compile(r"^\s*([A-Za-z_γα][A-Za-z0-9_γα]*)\s*=\s*(-?)\s*convert\(\s*T2?\s*,\s*([-+0-9.eE]+)\s*\)\s*(#.*)?$")


def parse_function(path: Path, fname: str):
    lines = path.read_text().splitlines()
    start = None
    for i, ln in enumerate(lines):
        if re.match(rf"^function {fname}\(", ln):
            start = i
            break
    if start is None:
        raise SystemExit(f"{fname} not found in {path}")
    out = []
    end = start
    for j in range(start + 1, len(lines)):
        ln = lines[j]
        if ln.startswith("end"):
            end = j
            break
        m = ASSIGN.match(ln)
        if m:
            name = m.group(1).replace("γ", "gamma").replace("α", "alpha")
            v = float(m.group(3))
            out.append((name, -v if m.group(2) else v))  # `-convert(T, x)`: negation is exact
    return out, start + 1, end + 1


def f32_literal(x: float) -> str:
    v = float(np.float32(np.float64(x)))
    s = repr(v)
    if "e" not in s and "." not in s:
        s += ".0"
    return s + "f"


# tables whose stage sums the fast-mode kernels evaluate two state components at a time
PACKED = ("vern7", "vern9")


def main():
    ref = Path(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
    oracle_lines = [
        "/* Generated by oracle/gen_tableaus.py -- do not edit.",
        " * FP64 coefficient literals of DiffEqGPU.jl's tableaus (see per-table citations).",
        " * Oracle (test infrastructure) copy; the kernels get the same numbers in tableaus_gen.cuh. */",
        "#pragma once",
        "",
    ]
    dev_lines = [
        "// Generated by oracle/gen_tableaus.py -- do not edit.",
        "// Method coefficients (Verner 7(6) and 9(8), Rodas5P, Rodas4, Kvaerno3/5) rounded once from their published FP64",
        "// values to FP32, exactly as Julia's convert(Float32, ::Float64) does in the reference",
        "// (see per-table citations).  They live in constant memory and are read as",
        "// constant-bank operands by the stage arithmetic.",
        "#pragma once",
        "",
    ]
    for tab, rel, fname in TABLES:
        entries, l0, l1 = parse_function(ref / rel, fname)
        entries = entries + derived(tab, entries)
        cite = f"{rel}:{l0}-{l1} ({fname})"
        names = [n for n, _ in entries]
        oracle_lines.append(f"/* {cite} */")
        oracle_lines.append("enum {")
        for n in names:
            oracle_lines.append(f"  OR_{tab.upper()}_{n},")
        oracle_lines.append(f"  OR_{tab.upper()}_COUNT")
        oracle_lines.append("};")
        oracle_lines.append(f"static const double OR_{tab.upper()}[OR_{tab.upper()}_COUNT] = {{")
        for n, v in entries:
            oracle_lines.append(f"  {v!r}, /* {n} */")
        oracle_lines.append("};")
        oracle_lines.append("")
        dev_lines.append(f"// {cite}")
        dev_lines.append("enum {")
        for n in names:
            dev_lines.append(f"  {tab.upper()}_{n},")
        dev_lines.append(f"  {tab.upper()}_COUNT")
        dev_lines.append("};")
        dev_lines.append(f"__constant__ float c_{tab}[{tab.upper()}_COUNT] = {{")
        for n, v in entries:
            dev_lines.append(f"  {f32_literal(v)}, // {n}")
        dev_lines.append("};")
        if tab in PACKED:
            # the same values as duplicated pairs, for the packed FP32 stage sums of fast mode
            dev_lines.append("#if DEGPU_PACKED_TABLES")
            dev_lines.append(f"__constant__ float2 c_{tab}_2[{tab.upper()}_COUNT] = {{")
            for n, v in entries:
                dev_lines.append(f"  {{{f32_literal(v)}, {f32_literal(v)}}}, // {n}")
            dev_lines.append("};")
            dev_lines.append("#endif")
        dev_lines.append("")
    (REPO / "oracle" / "tableaus_gen.h").write_text("\n".join(oracle_lines) + "\n")
    (REPO / "diffeqgpu.jl_gb300" / "csrc" / "device" / "tableaus_gen.cuh").write_text("\n".join(dev_lines) + "\n")
    print("wrote oracle/tableaus_gen.h and diffeqgpu.jl_gb300/csrc/device/tableaus_gen.cuh")


if __name__ == "__main__":
    main()
