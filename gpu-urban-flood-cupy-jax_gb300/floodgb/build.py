"""Build ``libfloodgb.so`` (the CUDA kernels + C ABI) in-tree with nvcc.

Kernels are compiled for sm_103a only (``-gencode arch=compute_103a,code=sm_103a``);
the drainage translation unit with ``-fmad=false`` (see ``csrc/fl_device.cuh``);
host sources are compiled by g++.  Objects go to ``gpu-urban-flood-cupy-jax_gb300/_build`` and the library to
``floodgb/_lib``.  Translation units compile in parallel; an up-to-date
library is not rebuilt.
"""

from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = ROOT / "csrc"
BUILD = ROOT / "_build"
LIB_DIR = PKG / "_lib"
LIB = LIB_DIR / "libfloodgb.so"
INCLUDE = ROOT.parent / "include"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> Path:
    env = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if env:
        return Path(env)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    return Path("/usr/local/cuda")


def _sources():
    cu = sorted(CSRC.glob("*.cu"))
    cpp = sorted(CSRC.glob("*.cpp"))
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))
    return cu, cpp, headers


def _up_to_date(target: Path, deps) -> bool:
    if not target.exists():
        return False
    t = target.stat().st_mtime
    return all(d.stat().st_mtime <= t for d in deps)


def build_library(force: bool = False, verbose: bool = False) -> Path:
    cu, cpp, headers = _sources()
    if not force and _up_to_date(LIB, list(cu) + list(cpp) + list(headers) + [Path(__file__)]):
        return LIB
    cuda = _cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    BUILD.mkdir(parents=True, exist_ok=True)
    LIB_DIR.mkdir(parents=True, exist_ok=True)
    inc = [f"-I{CSRC}", f"-I{INCLUDE}", f"-I{cuda / 'include'}"]
    jobs = []
    for src in cu:
        obj = BUILD / (src.stem + ".o")
        # the drainage kernels evaluate the same request/transfer at several call
        # sites and rely on uncontracted arithmetic for bit-identical results
        fmad = "-fmad=false" if src.stem in ("fl_drainage", "fl_inertial") else "-fmad=true"
        cmd = [nvcc, "-c", str(src), "-o", str(obj), *ARCH, "-O3", "-lineinfo", "-std=c++17", fmad,
               "-Xcompiler", "-fPIC,-fvisibility=hidden", "-Xptxas", "-v" if verbose else "-O3", *inc]
        jobs.append((obj, cmd))
    for src in cpp:
        obj = BUILD / (src.stem + ".o")
        cmd = ["g++", "-c", str(src), "-o", str(obj), "-O2", "-std=c++17", "-fPIC", "-fvisibility=hidden",
               "-Wall", "-Wno-unused-function", *inc]
        jobs.append((obj, cmd))

    def run(job):
        obj, cmd = job
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
        return res.stdout + res.stderr

    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as pool:
        logs = list(pool.map(run, jobs))
    if verbose:
        for log in logs:
            if log.strip():
                print(log)
    tmp = LIB.with_suffix(f".{os.getpid()}.tmp")
    link = [nvcc, "-shared", *ARCH, "-o", str(tmp), *[str(o) for o, _ in jobs], "-cudart", "static",
            "-Xlinker", "--exclude-libs,ALL"]
    res = subprocess.run(link, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(link)}\n{res.stdout}\n{res.stderr}")
    tmp.replace(LIB)
    return LIB


if __name__ == "__main__":
    import sys

    print(build_library(force="--force" in sys.argv, verbose="-v" in sys.argv))
