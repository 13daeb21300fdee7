"""Recipe that compiles the reference `symbolic_torch` extension from its own sources.

Test infrastructure only.  The sources are compiled where they lie under the
reference checkout (never copied); every output goes to ``oracle/_ref/``, which is
git-ignored.  The result is importable as the package ``symbolic_torch`` through
:func:`load_reference`, whose Python files are read from the reference checkout
and whose ``_C`` extension comes from ``oracle/_ref/``.

It is used in the development container to pin the C restatement in
``oracle/sr_oracle.c`` against the reference's own CPU path and to write the
golden fixtures under ``tests/golden/``.  The reference's CUDA sources are built
too (the extension cannot link without them) for sm_100; they are never run.

Usage:  python oracle/build_ref.py [REFERENCE_ROOT]
"""
from __future__ import annotations

import importlib.machinery
import importlib.util
import os
import sys
import types

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
DEFAULT_REF = "/root/reference"

# The reference's extension sources (setup.py lists the same eight files).
_SOURCES = [
    "src/main.cpp",
    "src/evaluation_kernels_cuda.cu",
    "src/evaluation_kernels_cpu.cpp",
    "src/symbolic_evaluation.cpp",
    "src/pcfg.cpp",
    "src/pcfg_cpu.cpp",
    "src/pcfg_cuda.cu",
    "src/utils.cpp",
]


def reference_root() -> str | None:
    root = os.environ.get("SR_REFERENCE_ROOT", DEFAULT_REF)
    return root if os.path.isfile(os.path.join(root, "src", "main.cpp")) else None


def _built_so() -> str | None:
    if not os.path.isdir(OUT):
        return None
    for f in os.listdir(OUT):
        if f.startswith("_C") and f.endswith(".so"):
            return os.path.join(OUT, f)
    return None


def build(ref_root: str | None = None, verbose: bool = False) -> str | None:
    """Compile the reference extension into ``oracle/_ref``; return the .so path.

    Returns None when the reference checkout is absent (e.g. on the GPU host).
    Skips the compile when the .so is newer than every source.
    """
    ref_root = ref_root or reference_root()
    if ref_root is None:
        return None
    srcs = [os.path.join(ref_root, s) for s in _SOURCES]
    so = _built_so()
    if so is not None:
        newest = max(os.path.getmtime(s) for s in srcs)
        if os.path.getmtime(so) >= newest:
            return so
    os.makedirs(OUT, exist_ok=True)
    os.environ.setdefault("TORCH_CUDA_ARCH_LIST", "10.0")
    from torch.utils.cpp_extension import load

    load(
        name="_C",
        sources=srcs,
        extra_include_paths=[os.path.join(ref_root, "include")],
        extra_cflags=["-O2", "-fopenmp"],
        extra_cuda_cflags=["-O2", "-Xcompiler", "-fopenmp", "--extended-lambda"],
        extra_ldflags=["-fopenmp"],
        build_directory=OUT,
        verbose=verbose,
        is_python_module=True,
    )
    return _built_so()


def build_error_messages(ref_root: str | None = None) -> str | None:
    """Compile ``oracle/ref_error_messages.cpp`` against the reference's
    ``include/error_codes.h`` (where it lies) into ``oracle/_ref/``; return the
    binary's path, or None without the reference checkout."""
    import subprocess
    ref_root = ref_root or reference_root()
    if ref_root is None:
        return None
    os.makedirs(OUT, exist_ok=True)
    exe = os.path.join(OUT, "ref_error_messages")
    src = os.path.join(HERE, "ref_error_messages.cpp")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ref_root, "include"), src, "-o", exe], check=True)
    return exe


def load_reference(ref_root: str | None = None) -> types.ModuleType:
    """Import the reference package ``symbolic_torch`` (Python files from the
    reference checkout, ``_C`` from ``oracle/_ref``)."""
    if "symbolic_torch" in sys.modules:
        return sys.modules["symbolic_torch"]
    ref_root = ref_root or reference_root()
    so = build(ref_root)
    if ref_root is None or so is None:
        raise RuntimeError("reference checkout not available")
    import torch  # noqa: F401  (loads libc10/libtorch for the extension)

    pkg_dir = os.path.join(ref_root, "symbolic_torch")
    # Load _C first under its package-qualified name.
    loader = importlib.machinery.ExtensionFileLoader("symbolic_torch._C", so)
    spec_c = importlib.util.spec_from_file_location("symbolic_torch._C", so, loader=loader)
    spec = importlib.util.spec_from_file_location(
        "symbolic_torch", os.path.join(pkg_dir, "__init__.py"),
        submodule_search_locations=[pkg_dir, OUT])
    pkg = importlib.util.module_from_spec(spec)
    sys.modules["symbolic_torch"] = pkg
    mod_c = importlib.util.module_from_spec(spec_c)
    sys.modules["symbolic_torch._C"] = mod_c
    spec_c.loader.exec_module(mod_c)
    spec.loader.exec_module(pkg)
    return pkg


if __name__ == "__main__":
    path = build(sys.argv[1] if len(sys.argv) > 1 else None, verbose=True)
    print(path if path else "reference checkout not found; nothing built")
