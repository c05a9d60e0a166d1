"""The code-specialised decoder kernels: their generated CUDA source for
circulant codes compiles for sm_103a with NVRTC (CPU only: compilation
needs no device), and CSR schedules have none.  GPU parity of the
specialised kernels against the table-driven ones is in
``test_gpu_ldpc.py``."""

from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np
import pytest

import oracle
from commkit_gb300 import _lib
from commkit_gb300 import workloads as W
from commkit_gb300.build import JIT_HEADERS as HEADERS
from tests.conftest import GOLDEN

CSRC = Path(__file__).resolve().parents[1] / "commkit_gb300" / "csrc"


def _nvrtc():
    for name in ("libnvrtc.so.13", "/usr/local/cuda/lib64/libnvrtc.so.13"):
        try:
            return ctypes.CDLL(name)
        except OSError:
            continue
    pytest.skip("NVRTC is not installed")


def _schedule(checks, variables, m, n):
    row_ptr, cols, layer_ptr = oracle.schedule(checks, variables, m, n)
    return row_ptr.astype(np.int32), cols.astype(np.int32), layer_ptr.astype(np.int32)


def source(row_ptr, cols, layer_ptr, m, n, form: int = 0) -> str:
    lib = _lib.lib()
    length = ctypes.c_size_t()
    args = (row_ptr.ctypes.data, cols.ctypes.data, layer_ptr.ctypes.data, m, n, layer_ptr.size - 1, form)
    _lib.check(lib.ck_ldpc_specialised_source(*args, None, 0, ctypes.byref(length)), "source size")
    buf = ctypes.create_string_buffer(length.value + 1)
    _lib.check(lib.ck_ldpc_specialised_source(*args, buf, len(buf), ctypes.byref(length)), "source")
    return buf.value.decode()


def compile_nvrtc(src: str) -> tuple[int, str]:
    nv = _nvrtc()
    names = [h.encode() for h in HEADERS]
    bodies = [(CSRC / h).read_bytes() for h in HEADERS]
    prog = ctypes.c_void_p()
    st = nv.nvrtcCreateProgram(ctypes.byref(prog), src.encode(), b"ck_ldpc_code.cu", len(HEADERS),
                               (ctypes.c_char_p * len(HEADERS))(*bodies), (ctypes.c_char_p * len(HEADERS))(*names))  # fmt: skip
    assert st == 0
    opts = [b"-arch=sm_103a", b"-std=c++17", b"-fmad=false"]
    st = nv.nvrtcCompileProgram(prog, len(opts), (ctypes.c_char_p * len(opts))(*opts))
    n = ctypes.c_size_t()
    nv.nvrtcGetProgramLogSize(prog, ctypes.byref(n))
    log = ctypes.create_string_buffer(n.value)
    nv.nvrtcGetProgramLog(prog, log)
    nv.nvrtcDestroyProgram(ctypes.byref(prog))
    return st, log.value.decode(errors="replace")


@pytest.mark.parametrize("name", ["A", "B", "C", "pon"])
def test_specialised_source_compiles(name):
    if name == "pon":
        g = np.load(GOLDEN / "ldpc_golden.npz")
        m, n = int(g["pon_m"]), int(g["pon_N"])
        sched = _schedule(g["pon_checks"], g["pon_variables"], m, n)
    else:
        spec = W.CODES[name]
        checks, variables = W.lift(spec.base(), spec.z)
        m, n = spec.mb * spec.z, spec.nb * spec.z
        sched = _schedule(checks, variables, m, n)
    src = source(*sched, m, n)
    # one row body per base row (Z rows each), one barrier per layer, two kernels
    bodies = src.count("st.template row_cols<")
    assert bodies > 0 and m % bodies == 0
    assert src.count("ck::group_sync(bar, T);") == sched[2].size - 1
    assert "ck_ldpc_code_r0" in src and "ck_ldpc_code_r1" in src and "ck_ldpc_code_r2" in src
    assert "decode_body<EdgeMinSumState" in src
    st, log = compile_nvrtc(src)
    assert st == 0, log[:3000]
    mixed = source(*sched, m, n, form=1)
    assert "ck_ldpc_mixed_code" in mixed and "CodeProgram0" in mixed
    st, log = compile_nvrtc(mixed)
    assert st == 0, log[:3000]
    # Two threads per row slot: every row body once, split between the parts.
    split = source(*sched, m, n, form=2)
    assert "kParts = 2" in split and split.count("st.template row_cols<") == bodies
    st, log = compile_nvrtc(split)
    assert st == 0, log[:3000]
    # One message per edge in shared memory (CK_LDPC_PLACE_EDGES).
    edges = source(*sched, m, n, form=3)
    assert ", true>(K, smem" in edges and "if (K.r_smem)" not in edges
    st, log = compile_nvrtc(edges)
    assert st == 0, log[:3000]


def test_csr_schedule_has_no_specialised_source():
    g = np.load(GOLDEN / "ldpc_golden.npz")
    m, n = int(g["dvbs2s_m"]), int(g["dvbs2s_N"])
    sched = _schedule(g["dvbs2s_checks"], g["dvbs2s_variables"], m, n)
    with pytest.raises(ValueError, match="circulant"):
        source(*sched, m, n)
