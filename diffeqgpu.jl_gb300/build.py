"""Build libdegpu.so in-tree (nvcc for sm_103a; no cmake).

Steps:
  1. embed the device sources (csrc/device/*.cuh|.h) and the built-in models
     (csrc/models/*.cuh) as string tables, so NVRTC needs no files at run time;
  2. compile and link the host library + the ahead-of-time kernels with nvcc;
  3. (check=True) compile the stepper/driver templates once per driver with nvcc
     -Xptxas -v, so that device-code errors surface at build time.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "degpu" / "libdegpu.so"
REPO = PKG.parent
CUDA = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA / "bin" / "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _c_string(text: str) -> str:
    out = []
    for line in text.splitlines(keepends=True):
        esc = line.replace("\\", "\\\\").replace('"', '\\"').replace("\n", "\\n")
        out.append(f'"{esc}"')
    return "\n".join(out) if out else '""'


def embed() -> Path:
    BUILD.mkdir(exist_ok=True)
    headers = sorted((CSRC / "device").glob("*.cuh")) + sorted((CSRC / "device").glob("*.h"))
    models = sorted((CSRC / "models").glob("*.cuh"))
    lines = ["// generated by build.py -- device sources for NVRTC", "#include <stddef.h>",
             "struct degpu_embedded_file { const char* name; const char* text; };",
             "struct degpu_embedded_model { const char* name; int n, p, flags; const char* text; };",
             'extern "C" const degpu_embedded_file degpu_embedded_headers[] = {']
    for h in headers:
        lines.append(f'  {{"{h.name}", {_c_string(h.read_text())}}},')
    lines.append("};")
    lines.append(f'extern "C" const int degpu_embedded_nheaders = {len(headers)};')
    lines.append('extern "C" const degpu_embedded_model degpu_embedded_models[] = {')
    for m in models:
        text = m.read_text()
        tag = text.splitlines()[0].split()
        assert tag[1] == "degpu-model:", m
        name, n, p, fl = tag[2], int(tag[3]), int(tag[4]), int(tag[5])
        lines.append(f'  {{"{name}", {n}, {p}, {fl}, {_c_string(text)}}},')
    lines.append("};")
    lines.append(f'extern "C" const int degpu_embedded_nmodels = {len(models)};')
    out = BUILD / "embedded.cpp"
    new = "\n".join(lines) + "\n"
    if not out.exists() or out.read_text() != new:
        out.write_text(new)
    return out


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def compile_lib(verbose: bool = False) -> Path:
    emb = embed()
    srcs = [CSRC / "degpu.cpp", emb] + sorted(CSRC.glob("*.cu"))
    inc = ["-I", str(REPO / "include"), "-I", str(CSRC), "-I", str(CSRC / "device")]
    objs = []

    def obj(src: Path):
        o = BUILD / (src.stem + ".o")
        deps = [src] + list((CSRC / "device").glob("*")) + [REPO / "include" / "degpu.h"]
        if o.exists() and all(o.stat().st_mtime >= d.stat().st_mtime for d in deps):
            return o, ""
        cmd = [NVCC, "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC", *inc, "-c", str(src), "-o", str(o)]
        if src.suffix == ".cu":
            cmd += ["-Xptxas", "-v"]
        return o, _run(cmd)

    with ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        for o, log in ex.map(obj, srcs):
            objs.append(o)
            if verbose and log:
                print(log)
    LIB.parent.mkdir(exist_ok=True)
    link = [NVCC, "-shared", *ARCH, "-o", str(LIB), *map(str, objs),
            "-L", str(CUDA / "lib64"), "-lnvrtc",
            "-Xlinker", f"-rpath={CUDA / 'lib64'}"]
    _run(link)
    return LIB


CHECKS = [  # (alg, driver, time type, parity, model, extra defines) compiled by the build check
    (0, 0, "float", 1, "lorenz", ""), (0, 1, "double", 0, "lorenz", ""), (0, 2, "double", 0, "lorenz", ""),
    (1, 2, "double", 0, "lorenz", ""), (2, 2, "double", 0, "lorenz", ""), (3, 2, "double", 0, "lorenz", ""),
    (3, 1, "double", 1, "lorenz", ""), (5, 2, "double", 0, "lorenz", ""), (6, 2, "double", 0, "lorenz", ""),
    (8, 2, "double", 0, "lorenz", ""), (9, 1, "float", 1, "lorenz", ""),
    # tstops + callbacks: continuous (bouncing ball) and discrete (decay) sets
    (0, 2, "double", 0, "ball", "-DDEGPU_NCCB=2 -DDEGPU_TSTOPS=1"),
    # SDE driver: Euler-Maruyama and SIEA on geometric Brownian motion
    (4, 3, "float", 1, "gbm", ""), (7, 3, "double", 0, "gbm", ""),
    # mass matrix (Robertson DAE)
    (2, 1, "float", 1, "robertson_dae", "-DDEGPU_MASS=1"), (3, 2, "double", 0, "robertson_dae", "-DDEGPU_MASS=1"),
    (1, 0, "float", 1, "decay", "-DDEGPU_NDCB=2 -DDEGPU_TSTOPS=1"),
]
MODEL_DIMS = {"lorenz": (3, 3), "ball": (2, 1), "decay": (1, 1), "gbm": (1, 2), "robertson_dae": (3, 3)}


def check_kernels(verbose: bool = False) -> list[str]:
    """Compile representative kernel instantiations with nvcc; returns ptxas lines."""
    BUILD.mkdir(exist_ok=True)

    def one(c):
        alg, drv, tt, par, model, extra = c
        n, p = MODEL_DIMS[model]
        tag = f"{alg}_{drv}_{tt}_{par}_{model}_{len(extra)}"
        tu = BUILD / f"kernel_check_{tag}.cu"
        tu.write_text(f'#include "degpu_prelude.cuh"\n#include "{model}.cuh"\n#include "degpu_kernels.cuh"\n')
        cmd = [NVCC, "-std=c++17", *ARCH, "-Xptxas", "-v", "-c", str(tu), "-o", os.devnull,
               "-I", str(CSRC / "device"), "-I", str(CSRC / "models"),
               f"-DDEGPU_N={n}", f"-DDEGPU_P={p}", f"-DDEGPU_ALG={alg}", f"-DDEGPU_DRIVER={drv}", f"-DDEGPU_TT={tt}",
               f"-DDEGPU_PARITY={par}", "-DDEGPU_JAC=0", "-DDEGPU_TGRAD=0", "-DDEGPU_LINSOLVE_REFINE=1",
               f"-DDEGPU_TIME_DF={1 if tt == 'double' else 0}", *extra.split()]
        cmd += ["-fmad=false", "-prec-div=true", "-prec-sqrt=true"] if par else ["-prec-div=false", "-prec-sqrt=false"]
        log = _run(cmd)
        return [f"alg={alg} driver={drv} tt={tt} parity={par} {model} {extra}: {ln.strip()}"
                for ln in log.splitlines() if "registers" in ln]

    out = []
    with ThreadPoolExecutor(max_workers=len(CHECKS)) as ex:
        for lines in ex.map(one, CHECKS):
            out += lines
    if verbose:
        print("\n".join(out))
    return out


def build(check: bool = True, verbose: bool = False) -> Path:
    lib = compile_lib(verbose)
    if check:
        check_kernels(verbose)
    return lib


if __name__ == "__main__":
    build(check="--no-check" not in sys.argv, verbose=True)
    print(LIB)
