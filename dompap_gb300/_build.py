"""Build the CUDA library ``libdompap_gpu.so`` in-tree for sm_103a.

``python -m dompap_gb300._build`` (or ``__graft_entry__.build()``) runs nvcc
once: the C ABI and the statically compiled kernels in ``csrc/dompap_gpu.cu``
are compiled for ``sm_103a`` and linked with NVRTC, which compiles the pair
kernels (``csrc/pair_kernels.cuh``) at run time for each SymPy pair potential.
The two ``.cuh`` sources NVRTC needs are embedded into the library as string
literals (``_build/dp_embedded.h``), so the ``.so`` is self-contained.

A second, optional nvcc pass compiles the pair kernels for a sample potential
(harmonic, LJ) to catch template errors without a GPU and to report registers
and spills (``-Xptxas -v``).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libdompap_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build dompap_gb300")
    return path


def _cuda_home(nvcc: str) -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def write_embedded() -> str:
    os.makedirs(BUILD, exist_ok=True)
    parts = []
    for name, sym in (("dp_common.cuh", "dp_src_common"), ("pair_kernels.cuh", "dp_src_pair"),
                      ("batch_kernels.cuh", "dp_src_batch"), ("mlp_common.cuh", "dp_src_mlp"),
                      ("dp_ff.cuh", "dp_src_ff"), ("dp_integrate.cuh", "dp_src_integrate"),
                      ("dp_umma.cuh", "dp_src_umma")):
        with open(os.path.join(CSRC, name)) as fh:
            text = fh.read()
        if ')DPSRC"' in text:
            raise RuntimeError(f"{name} contains the raw-string delimiter")
        # NVRTC sees the text after the configuration macros; drop '#pragma once'
        text = text.replace("#pragma once", "")
        parts.append(f'static const char {sym}[] = R"DPSRC({text})DPSRC";\n')
    out = os.path.join(BUILD, "dp_embedded.h")
    content = "// generated by dompap_gb300/_build.py — do not edit\n#pragma once\n" + "".join(parts)
    old = open(out).read() if os.path.exists(out) else None
    if old != content:
        with open(out, "w") as fh:
            fh.write(content)
    return out


def build_library(verbose: bool = False) -> str:
    nvcc = _nvcc()
    cuda = _cuda_home(nvcc)
    write_embedded()
    src = os.path.join(CSRC, "dompap_gpu.cu")
    tmp = LIB + ".tmp"
    cmd = [
        nvcc, *ARCH, "-O3", "-std=c++17", "-lineinfo", "-shared", "-Xcompiler", "-fPIC",
        "-I", os.path.join(REPO, "include"), "-I", CSRC, "-I", BUILD,
        src, "-o", tmp,
        "-L", os.path.join(cuda, "lib64"), "-lnvrtc",
        "-Xlinker", "-rpath," + os.path.join(cuda, "lib64"),
    ]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr)
    if verbose:
        sys.stdout.write(res.stdout + res.stderr)
    os.replace(tmp, LIB)
    return LIB


SAMPLE_POTENTIAL = """
template <typename R> __device__ __forceinline__ R dp_pair_u(R s, R) { R t = R(1) - s; return t * t; }
template <typename R> __device__ __forceinline__ R dp_pair_f(R s, R) { return R(2) * (R(1) - s); }
template <typename R> __device__ __forceinline__ R dp_pair_c(R s, R) { return R(2); }
"""


def check_pair_kernels(verbose: bool = True) -> None:
    """nvcc-compile the NVRTC template for every (D, precision, mode) to catch errors offline."""
    nvcc = _nvcc()
    write_embedded()
    with open(os.path.join(CSRC, "dp_common.cuh")) as fh:
        common = fh.read()
    with open(os.path.join(CSRC, "pair_kernels.cuh")) as fh:
        pair = fh.read()
    with open(os.path.join(CSRC, "batch_kernels.cuh")) as fh:
        batch = fh.read()
    with open(os.path.join(CSRC, "dp_ff.cuh")) as fh:
        ffsrc = fh.read()
    with open(os.path.join(CSRC, "dp_integrate.cuh")) as fh:
        integ = fh.read()
    for dim in (2, 3, 4):
        for real, is_float in (("double", 0), ("float", 1)):
            for pmode in (0, 1, 2):
                src = (f"#define DP_DIM {dim}\n#define DP_REAL {real}\n#define DP_REAL_IS_FLOAT {is_float}\n"
                       f"#define DP_PMODE {pmode}\n#define DP_SIGMA_ONE {int(pmode == 0)}\n"
                       f"#define DP_EPS_ONE {int(pmode == 0)}\n#define DP_FF {1 - is_float}\n#include <cstdint>\n"
                       + common + integ + (ffsrc if not is_float else "") + SAMPLE_POTENTIAL + pair
                       + (batch if is_float and pmode == 0 else ""))
                path = os.path.join(BUILD, f"pair_check_{dim}_{real}_{pmode}.cu")
                with open(path, "w") as fh:
                    fh.write(src)
                cmd = [nvcc, *ARCH, "-O3", "-std=c++17", "-c", path, "-o", path + ".o"]
                if verbose and pmode == 0:
                    cmd.insert(1, "-Xptxas=-v")
                res = subprocess.run(cmd, capture_output=True, text=True)
                if res.returncode != 0:
                    raise RuntimeError("pair kernel check failed:\n" + res.stdout + res.stderr)
                if verbose and pmode == 0:
                    lines = [ln for ln in (res.stdout + res.stderr).splitlines() if "registers" in ln or "spill" in ln]
                    print(f"[D={dim} {real}]", *lines, sep="\n  ")


if __name__ == "__main__":
    print(build_library(verbose="-v" in sys.argv))
    if "--check" in sys.argv:
        check_pair_kernels()
