"""Build recipe for the reference's own CUDA extension (sxyu/svox2 ``svox2.csrc``) — TEST
INFRASTRUCTURE, never part of the product.

The GPU parity tests use the reference's compiled kernels as a second checker beside the CPU
oracle: on the same inputs, at the default thresholds, they compare this library's colours,
gradients and masks (and the MSI background, whose CUDA semantics the reference's pure-PyTorch
path does not share) with what the reference's extension computes.  ``bench.py --config refgpu``
times the same extension's training step as the plain-FP32 GPU form.

Two steps:
  * ``stage(ref_root)`` copies the reference's extension sources (``svox2/csrc``: the .cu/.cpp
    files and ``include/``) and its Python package files, unmodified, into ``oracle/_ref/src``.
    That folder is git-ignored: it is not part of the repository, but it travels with the
    working tree to machines that have no reference checkout, where the extension must be
    compiled for their own architecture.
  * ``build()`` compiles the staged sources with nvcc/g++ against the installed PyTorch into
    ``oracle/_ref/svox2_ref_csrc.<machine>.so`` (module name ``svox2_ref_csrc``, so it cannot
    shadow anything).  One object per source, in parallel, as the reference's own setup.py lists them
    (``setup.py:39-49``); the flags are PyTorch's CUDAExtension defaults with the GB300
    architecture.  No cmake, no ninja.

``load()`` imports the built module, or returns None when it is not there.
"""
from __future__ import annotations

import concurrent.futures as _fut
import importlib.util
import os
import platform
import shutil
import subprocess
import sys
import sysconfig
from pathlib import Path

ORACLE_DIR = Path(__file__).resolve().parent
REF_DIR = ORACLE_DIR / "_ref"
SRC_DIR = REF_DIR / "src"
MODULE = "svox2_ref_csrc"
# objects and module per host architecture: the working tree travels between x86 and Arm hosts
BUILD_DIR = REF_DIR / f"build-{platform.machine()}"
LIB = REF_DIR / f"{MODULE}.{platform.machine()}.so"
DEFAULT_REF_ROOT = Path("/root/reference")

# svox2/csrc sources of the extension, as setup.py:39-49 lists them
CSRC = ["svox2.cpp", "svox2_kernel.cu", "render_lerp_kernel_cuvol.cu", "render_lerp_kernel_nvol.cu",
        "render_svox1_kernel.cu", "misc_kernel.cu", "loss_kernel.cu", "optim_kernel.cu"]
PY = ["__init__.py", "defs.py", "svox2.py", "utils.py", "version.py"]

_module = None


def staged() -> bool:
    return all((SRC_DIR / "svox2" / "csrc" / f).exists() for f in CSRC)


def stage(ref_root: Path = DEFAULT_REF_ROOT) -> bool:
    """Copy the reference's extension sources and Python files into oracle/_ref/src.
    Returns False (and does nothing) when ref_root is not a reference checkout."""
    ref_root = Path(ref_root)
    src = ref_root / "svox2"
    if not all((src / "csrc" / f).exists() for f in CSRC):
        return False
    dst = SRC_DIR / "svox2"
    (dst / "csrc" / "include").mkdir(parents=True, exist_ok=True)
    for f in CSRC:
        _copy_if_newer(src / "csrc" / f, dst / "csrc" / f)
    for h in sorted((src / "csrc" / "include").iterdir()):
        if h.is_file():
            _copy_if_newer(h, dst / "csrc" / "include" / h.name)
    for f in PY:
        if (src / f).exists():
            _copy_if_newer(src / f, dst / f)
    return True


def _copy_if_newer(a: Path, b: Path) -> None:
    if not b.exists() or b.stat().st_mtime < a.stat().st_mtime or b.stat().st_size != a.stat().st_size:
        shutil.copyfile(a, b)


def _torch_paths():
    import torch
    root = Path(torch.__file__).resolve().parent
    inc = [root / "include", root / "include" / "torch" / "csrc" / "api" / "include"]
    return root, inc, root / "lib", bool(torch._C._GLIBCXX_USE_CXX11_ABI)


def _cuda_home() -> Path:
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    return Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))


def build(force: bool = False, verbose: bool = False) -> Path | None:
    """Compile the staged sources into oracle/_ref/svox2_ref_csrc.so.  Returns its path, or
    None when nothing is staged or no CUDA toolkit is present."""
    if not staged():
        return None
    cuda = _cuda_home()
    nvcc = cuda / "bin" / "nvcc"
    if not nvcc.exists():
        return None
    _, tinc, tlib, abi = _torch_paths()
    csrc = SRC_DIR / "svox2" / "csrc"
    incs = [csrc / "include", *tinc, cuda / "include", Path(sysconfig.get_paths()["include"])]
    defs = [f"-DTORCH_EXTENSION_NAME={MODULE}", "-DTORCH_API_INCLUDE_EXTENSION_H",
            f"-D_GLIBCXX_USE_CXX11_ABI={int(abi)}"]
    inc_flags = [f for p in incs for f in ("-isystem", str(p))]
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    deps = sorted((csrc / "include").iterdir())
    jobs, objs = [], []
    for f in CSRC:
        s = csrc / f
        o = BUILD_DIR / (s.stem + ".o")
        objs.append(o)
        if not force and o.exists() and all(o.stat().st_mtime >= d.stat().st_mtime for d in [s, *deps]):
            continue
        if s.suffix == ".cu":
            cmd = [str(nvcc), *defs, *inc_flags, "-D__CUDA_NO_HALF_OPERATORS__", "-D__CUDA_NO_HALF_CONVERSIONS__",
                   "-D__CUDA_NO_BFLOAT16_CONVERSIONS__", "-D__CUDA_NO_HALF2_OPERATORS__", "--expt-relaxed-constexpr",
                   "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-w", "-c", str(s), "-o", str(o)]
        else:
            cmd = ["g++", *defs, *inc_flags, "-O3", "-std=c++17", "-fPIC", "-w", "-c", str(s), "-o", str(o)]
        jobs.append(cmd)

    def run(cmd):
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"reference extension build failed ({' '.join(cmd[:1] + cmd[-3:])}):\n"
                               f"{res.stdout[-4000:]}\n{res.stderr[-4000:]}")
        return res.stdout + res.stderr

    if jobs:
        with _fut.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for out in ex.map(run, jobs):
                if verbose and out.strip():
                    print(out)
    if force or jobs or not LIB.exists() or any(o.stat().st_mtime > LIB.stat().st_mtime for o in objs):
        tmp = LIB.with_suffix(".so.tmp")
        run(["g++", "-shared", *map(str, objs), f"-L{tlib}", "-lc10", "-lc10_cuda", "-ltorch", "-ltorch_cpu",
             "-ltorch_cuda", "-ltorch_python", f"-L{cuda / 'lib64'}", "-lcudart", f"-Wl,-rpath,{tlib}",
             "-o", str(tmp)])
        os.replace(tmp, LIB)
    return LIB


def load():
    """The reference's extension module (svox2_ref_csrc), or None when it has not been built
    for this machine.  PyTorch is imported first: the module links against it."""
    global _module
    if _module is not None:
        return _module
    if not LIB.exists():
        return None
    import torch  # noqa: F401
    spec = importlib.util.spec_from_file_location(MODULE, str(LIB))
    mod = importlib.util.module_from_spec(spec)
    try:
        spec.loader.exec_module(mod)
    except ImportError:
        return None   # built for another machine (the x86 file on an Arm host, or the reverse)
    sys.modules[MODULE] = mod
    _module = mod
    return mod


def import_reference_package(with_extension: bool = True):
    """The reference's own Python package (sxyu/svox2 ``svox2``, staged unmodified into
    oracle/_ref/src), bound to its own compiled extension when with_extension and the extension
    is built for this machine; otherwise it runs its pure-PyTorch path only (its ``_C`` is None).
    The package imports tqdm (a progress bar) at module level; where tqdm is not installed a
    pass-through stand-in is registered under that name.  Returns None when nothing is staged."""
    if not (SRC_DIR / "svox2" / "svox2.py").exists():
        return None
    if "svox2" in sys.modules:
        return sys.modules["svox2"]
    try:
        import tqdm  # noqa: F401
    except ImportError:
        import types

        stub = types.ModuleType("tqdm")
        stub.tqdm = lambda it=None, *a, **k: it
        sys.modules["tqdm"] = stub
    if with_extension:
        mod = load()
        if mod is not None:
            sys.modules["svox2.csrc"] = mod
    if str(SRC_DIR) not in sys.path:
        sys.path.insert(0, str(SRC_DIR))
    import warnings

    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        import svox2
    return svox2


if __name__ == "__main__":
    root = Path(sys.argv[1]) if len(sys.argv) > 1 else DEFAULT_REF_ROOT
    print("staged:", stage(root) or staged())
    print(build(verbose=True))
