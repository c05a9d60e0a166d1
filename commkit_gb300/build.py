"""In-tree build of ``libck_gb300.so``, the CUDA library behind the package.

``python -m commkit_gb300.build`` compiles every ``csrc/*.cu`` / ``*.cpp``
for sm_103a only (``-gencode arch=compute_103a,code=sm_103a``), in parallel,
and links them against the shared CUDA runtime into
``commkit_gb300/_lib/libck_gb300.so``.  Objects go to ``commkit_gb300/_build``.
Beside it, ``csrc/python/ck_calls.cpp`` becomes the per-call CPython
extension over the installed torch (``_lib/ck_calls*.so``).
Rebuilds only what changed (sources or headers newer than the object).
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
import sysconfig
import warnings
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
SRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIB_DIR = PKG / "_lib"
LIB = LIB_DIR / "libck_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = [
    "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
    # Every float operation of the kernels rounds once, as the reference's
    # (explicit _rn intrinsics too; this keeps stray expressions honest).
    "-fmad=false", "--expt-relaxed-constexpr",
]  # fmt: skip


def nvcc() -> str:
    found = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(found).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build commkit_gb300")
    return found


# Kernel headers the code-specialised decoders are compiled from at run time
# (NVRTC): embedded in the library as strings.
JIT_HEADERS = ("ck_device.cuh", "ck_llr_axis.cuh", "ck_ldpc_kernel.cuh", "ck_ldpc_minsum.cuh", "ck_ldpc_mixed.cuh")
JIT_SOURCE = BUILD / "ck_jit_headers.cpp"


def _jit_headers() -> Path:
    """Writes the embedded-header source if a header changed since."""
    deps = [SRC / h for h in JIT_HEADERS]
    if _stale(JIT_SOURCE, deps):
        parts = ["// Written by commkit_gb300/build.py: NVRTC sources of the kernel headers.",
                 f"extern const int ck_jit_header_count = {len(JIT_HEADERS)};",
                 "extern const char* const ck_jit_header_names[] = {" + ", ".join(f'"{h}"' for h in JIT_HEADERS) + "};",
                 "extern const char* const ck_jit_header_sources[] = {"]  # fmt: skip
        for d in deps:
            text = d.read_text()
            if ')ckjit"' in text:
                raise RuntimeError(f"{d.name} holds the raw-string delimiter")
            parts.append('R"ckjit(' + text + ')ckjit",')
        parts.append("};")
        tmp = JIT_SOURCE.with_suffix(f".{os.getpid()}.tmp")
        tmp.write_text("\n".join(parts) + "\n")
        os.replace(tmp, JIT_SOURCE)
    return JIT_SOURCE


def _sources() -> list[Path]:
    return sorted([*SRC.glob("*.cu"), *SRC.glob("*.cpp")]) + [_jit_headers()]


def _headers() -> list[Path]:
    return [*SRC.glob("*.cuh"), *SRC.glob("*.h"), *INCLUDE.glob("*.h")]


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _compile(src: Path, verbose: bool) -> Path:
    obj = BUILD / (src.name + ".o")
    if not _stale(obj, [src, *_headers()]):
        return obj
    cmd = [nvcc(), *ARCH, *FLAGS, "-I", str(INCLUDE), "-I", str(SRC), "-c", str(src), "-o", str(obj)]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{res.stdout}\n{res.stderr}")
    if verbose and (res.stdout or res.stderr):
        print(res.stdout + res.stderr, file=sys.stderr)
    return obj


CALLS_SRC = SRC / "python" / "ck_calls.cpp"
CALLS = LIB_DIR / ("ck_calls" + (sysconfig.get_config_var("EXT_SUFFIX") or ".so"))


def build_calls() -> Path | None:
    """The per-call extension (``compute_llr``/``decode`` of torch tensors
    without ctypes), compiled against the installed torch's headers and
    libraries; None, with a warning, where those or Python's headers are
    missing or the compiler fails (the package then calls through ctypes)."""
    try:
        import torch
    except ImportError:
        return None
    tdir = Path(torch.__file__).resolve().parent
    py_inc = Path(sysconfig.get_paths()["include"])
    deps = [CALLS_SRC, INCLUDE / "commkit_gb300.h", tdir / "version.py"]
    if not _stale(CALLS, deps):
        return CALLS
    if not (py_inc / "Python.h").exists() or not (tdir / "include" / "ATen").is_dir():
        warnings.warn("Python or torch headers missing: the per-call extension is not built", stacklevel=2)
        return None
    cuda_inc = Path(nvcc()).resolve().parent.parent / "include"
    tmp = CALLS.with_suffix(f".{os.getpid()}.tmp")
    cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-fPIC", "-shared", "-Wall",
           f"-D_GLIBCXX_USE_CXX11_ABI={int(torch.compiled_with_cxx11_abi())}",
           "-I", str(py_inc), "-I", str(tdir / "include"), "-I", str(tdir / "include" / "torch" / "csrc" / "api" / "include"),
           "-I", str(cuda_inc), "-I", str(INCLUDE), str(CALLS_SRC), "-o", str(tmp),
           "-L", str(tdir / "lib"), "-lc10", "-lc10_cuda", "-ltorch_cpu", "-ltorch_python",
           f"-Wl,-rpath,{tdir / 'lib'}"]  # fmt: skip
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        warnings.warn(f"the per-call extension did not compile:\n{res.stderr[-4000:]}", stacklevel=2)
        return None
    os.replace(tmp, CALLS)
    return CALLS


def build(verbose: bool = False) -> Path:
    """Compile and link the library if anything changed; returns its path."""
    BUILD.mkdir(exist_ok=True)
    LIB_DIR.mkdir(exist_ok=True)
    srcs = _sources()
    with ThreadPoolExecutor(max_workers=min(8, len(srcs) + 1)) as pool:
        calls = pool.submit(build_calls)
        objs = list(pool.map(lambda s: _compile(s, verbose), srcs))
        calls.result()
    if _stale(LIB, objs):
        tmp = LIB.with_suffix(f".{os.getpid()}.tmp")
        # The shared CUDA runtime (soname libcudart.so.13): a process that has
        # loaded torch's copy reuses it, so both see one current device.
        cmd = [nvcc(), *ARCH, "-shared", "-cudart", "shared", "-Xlinker", "-rpath=/usr/local/cuda/lib64",
               "-o", str(tmp), *map(str, objs), "-ldl"]  # fmt: skip
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
