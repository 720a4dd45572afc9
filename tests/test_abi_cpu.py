"""CPU checks of the boundary: the C-ABI library loads without a GPU and
exports every entry point ``include/dompap_gpu.h`` declares; the ctypes
binding covers them; code generation output; failing loudly without a GPU."""
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import REPO

HEADER = os.path.join(REPO, "include", "dompap_gpu.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(dp_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from dompap_gb300 import _lib

    if not os.path.exists(_lib.LIB_PATH):
        from dompap_gb300 import _build

        _build.build_library()
    return _lib.load()


def test_library_exports_every_declared_symbol(lib):
    syms = declared_symbols()
    assert len(syms) >= 30
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", os.path.join(REPO, "dompap_gb300", "libdompap_gpu.so")],
                         capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (dp_[a-z0-9_]+)", out))
    assert set(syms) <= exported, sorted(set(syms) - exported)


def test_binding_covers_header(lib):
    from dompap_gb300 import _lib

    assert set(declared_symbols()) == set(_lib.exported_symbols())
    assert lib.dp_version() >= 100


def test_no_gpu_fails_loudly(lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from dompap_gb300 import Simulation
    from dompap_gb300._lib import DompapGPUError

    with pytest.raises(DompapGPUError):
        Simulation()


def test_codegen_sources():
    from dompap_gb300 import codegen

    src, rc = codegen.make_pair_source("4*(r**-12-r**-6)", 2.5)
    assert "dp_pair_u" in src and "dp_pair_f" in src and "dp_pair_c" in src and rc == 2.5
    assert " pow(" not in src and "(pow(" not in src  # integer powers become multiplication chains
    assert np.isclose(codegen.value_at_cut("4*(r**-12-r**-6)", 2.5), 4 * (2.5 ** -12 - 2.5 ** -6), rtol=1e-15)
    src, rc = codegen.make_pair_source("Harmonic repulsive", 99.0)
    assert rc == 1.0
    with pytest.raises(ValueError):
        codegen.make_pair_source("(1-r)**2 + x", 1.0)
    src, _ = codegen.make_pair_source("exp(-r)*cos(4*r) + (((1-r)**2)**(1/2))**(7/2)", 1.0)
    assert "exp(" in src and "cos(" in src


def test_generated_source_compiles_with_nvcc(tmp_path):
    """The NVRTC program (configuration macros + common header + generated
    potential + pair kernels) is valid CUDA for sm_103a."""
    from dompap_gb300 import _build, codegen

    src, _ = codegen.make_pair_source(
        "4*(r**-12-r**-6) + 0.5*exp(-(r-1.5)**2/0.02) + 0.1*cos(4*r)*exp(-r)", 3.0)
    common = open(os.path.join(_build.CSRC, "dp_common.cuh")).read()
    integ = open(os.path.join(_build.CSRC, "dp_integrate.cuh")).read()
    ff = open(os.path.join(_build.CSRC, "dp_ff.cuh")).read()
    pair = open(os.path.join(_build.CSRC, "pair_kernels.cuh")).read()
    prog = ("#define DP_DIM 3\n#define DP_REAL double\n#define DP_REAL_IS_FLOAT 0\n#define DP_PMODE 1\n"
            "#define DP_SIGMA_ONE 0\n#define DP_EPS_ONE 0\n#define DP_FF 1\n#include <cstdint>\n"
            + common + integ + ff + src + pair)
    path = tmp_path / "prog.cu"
    path.write_text(prog)
    res = subprocess.run([_build._nvcc(), *_build.ARCH, "-std=c++17", "-c", str(path), "-o", str(tmp_path / "p.o")],
                         capture_output=True, text=True)
    assert res.returncode == 0, res.stderr


def test_oracle_only_imported_by_checkers():
    """The product package never imports the oracle."""
    pkg = os.path.join(REPO, "dompap_gb300")
    for root, _, files in os.walk(pkg):
        for name in files:
            if name.endswith((".py", ".cu", ".cuh", ".h")):
                text = open(os.path.join(root, name)).read()
                assert "import oracle" not in text and "from oracle" not in text, name


@pytest.mark.parametrize("dim,precision,pmode,batch", [
    (d, p, 0, 0) for d in (2, 3, 4) for p in (0, 1, 2)] + [
    (3, 0, 1, 0), (3, 0, 2, 0), (3, 1, 1, 0)] + [
    (d, 1, 0, 1) for d in (2, 3, 4)])
def test_nvrtc_programs_compile(dim, precision, pmode, batch):
    """Every device program the library builds at run time (pair kernels, fused
    step, surrogate, batch) compiles with NVRTC for sm_103a — checked on the
    host through the library's own program assembly (no GPU needed)."""
    import ctypes

    from dompap_gb300 import _lib, codegen

    src, _ = codegen.make_pair_source("4*(r**-12-r**-6) + 0.5*exp(-(r-1.5)**2/0.02)", 2.5)
    size = ctypes.c_int64(0)
    rc = _lib.load().dp_nvrtc_check(dim, precision, pmode, batch, src.encode(), ctypes.byref(size))
    assert rc == 0, _lib.load().dp_last_error().decode()
    assert size.value > 10000


def _registers_by_kernel(dim):
    import ctypes
    import re

    from dompap_gb300 import _lib, codegen

    src, _ = codegen.make_pair_source("(1-r)**2", 1.0)
    buf = ctypes.create_string_buffer(1 << 18)
    size = ctypes.c_int64(0)
    rc = _lib.load().dp_nvrtc_resources(dim, 0, 0, 0, src.encode(), buf, len(buf), ctypes.byref(size))
    assert rc == 0, _lib.load().dp_last_error().decode()
    assert 0 < size.value <= len(buf)
    used = {}
    kernel = None
    for line in buf.value.decode().splitlines():
        m = re.search(r"entry function '(\w+)'", line)
        if m:
            kernel = m.group(1)
        m = re.search(r"Used (\d+) registers", line)
        if m and kernel:
            used[kernel] = int(m.group(1))
    return used


def test_nvrtc_resource_report():
    """The assembler's verbose report of a run-time program: every kernel's
    registers, spills and shared memory (the float64-parity fused step in 3-D
    is built for four resident 256-thread CTAs per SM, so at most 64
    registers; in 2-D for six, at most 40)."""
    used = _registers_by_kernel(3)
    assert {"dp_forces", "dp_step", "dp_energy", "dp_virial"} <= set(used)
    assert used["dp_step"] <= 64
    assert _registers_by_kernel(2)["dp_step"] <= 40


def test_nvrtc_cubin_cache(tmp_path, monkeypatch):
    """The on-disk cache of compiled pair programs: the first compile writes a
    file keyed by the program text, the second reads it instead of compiling,
    a damaged file is ignored and rewritten, another potential gets its own."""
    import ctypes
    import time

    from dompap_gb300 import _lib, codegen

    monkeypatch.setenv("DOMPAP_NVRTC_CACHE", str(tmp_path))
    lib = _lib.load()
    src, _ = codegen.make_pair_source("(1-r)**2", 1.0)

    def compile_once(source):
        size = ctypes.c_int64(0)
        t0 = time.perf_counter()
        assert lib.dp_nvrtc_check(3, 1, 0, 0, source.encode(), ctypes.byref(size)) == 0, lib.dp_last_error()
        return size.value, time.perf_counter() - t0

    size1, t_compile = compile_once(src)
    files = sorted(tmp_path.glob("*.dpcubin"))
    assert len(files) == 1 and files[0].read_bytes()[:8] == b"DPCUBIN1"
    size2, t_cached = compile_once(src)
    assert size2 == size1 and t_cached < 0.5 * t_compile
    files[0].write_bytes(b"not a cubin")
    size3, _ = compile_once(src)
    assert size3 == size1 and files[0].read_bytes()[:8] == b"DPCUBIN1"
    src_lj, _ = codegen.make_pair_source("4*(r**-12-r**-6)", 2.5)
    compile_once(src_lj)
    assert len(list(tmp_path.glob("*.dpcubin"))) == 2
