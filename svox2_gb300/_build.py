"""In-tree build of the CUDA library ``libsvox2_gb300.so`` (sm_103a only).

The library is compiled with nvcc directly (one object per ``csrc/*.cu``,
compiled in parallel, then linked with ``-shared``).  It has no Python or
PyTorch dependency: everything it exports is the C ABI declared in
``include/svox2_gb300.h``.
"""
from __future__ import annotations

import concurrent.futures as _fut
import os
import shutil
import subprocess
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
REPO_DIR = PKG_DIR.parent
CSRC_DIR = PKG_DIR / "csrc"
LIB_DIR = PKG_DIR / "lib"
LIB_PATH = LIB_DIR / "libsvox2_gb300.so"
BUILD_DIR = PKG_DIR / "_build"

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3",
    "-std=c++17",
    "-lineinfo",
    "-Xcompiler",
    "-fPIC",
    "--expt-relaxed-constexpr",
    "-Xptxas",
    "-warn-spills",
]


def nvcc_path() -> str:
    cand = shutil.which("nvcc")
    if cand:
        return cand
    home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    p = Path(home) / "bin" / "nvcc"
    if p.exists():
        return str(p)
    raise RuntimeError("nvcc not found: set CUDA_HOME or put nvcc on PATH")


def sources() -> list[Path]:
    return sorted(CSRC_DIR.glob("*.cu"))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False, extra_flags: list[str] | None = None) -> Path:
    """Compile ``csrc/*.cu`` into ``lib/libsvox2_gb300.so``; returns its path."""
    nvcc = nvcc_path()
    BUILD_DIR.mkdir(exist_ok=True)
    LIB_DIR.mkdir(exist_ok=True)
    headers = sorted(CSRC_DIR.glob("*.cuh")) + [REPO_DIR / "include" / "svox2_gb300.h"]
    flags = ARCH_FLAGS + NVCC_FLAGS + (extra_flags or [])
    jobs = []
    objs = []
    for src in sources():
        obj = BUILD_DIR / (src.stem + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            cmd = [nvcc, *flags, "-c", str(src), "-o", str(obj)]
            jobs.append(cmd)

    def run(cmd):
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed ({' '.join(cmd)}):\n{res.stdout}\n{res.stderr}")
        return res.stdout + res.stderr

    if jobs:
        with _fut.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for out in ex.map(run, jobs):
                if verbose and out.strip():
                    print(out)
    if force or jobs or _stale(LIB_PATH, objs):
        tmp = LIB_PATH.with_suffix(".so.tmp")
        run([nvcc, *ARCH_FLAGS, "-shared", *[str(o) for o in objs], "-o", str(tmp)])
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose=True))
