"""Build of libsphere_stereo_gb300.so: every csrc/*.cu compiled for sm_103a in parallel, then
linked into one shared library next to this file (the CUDA runtime is linked statically)."""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
LIBRARY = os.path.join(HERE, "libsphere_stereo_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
                     "--expt-relaxed-constexpr"]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build sphere_stereo_gb300")
    return path


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile (if anything changed) and return the path of the shared library."""
    os.makedirs(OBJ, exist_ok=True)
    headers = _headers()
    srcs = sources()
    objs = [os.path.join(OBJ, os.path.basename(s)[:-3] + ".o") for s in srcs]
    exe = nvcc()

    def compile_one(pair):
        src, obj = pair
        if not force and not _stale(obj, [src] + headers):
            return None
        tmp = f"{obj}.{os.getpid()}.tmp"
        cmd = [exe, *NVCC_FLAGS, "-c", src, "-o", tmp]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            return f"{' '.join(cmd)}\n{r.stdout}{r.stderr}"
        os.replace(tmp, obj)
        if verbose:
            print(r.stderr, end="")
        return None

    with ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 1))) as pool:
        errors = [e for e in pool.map(compile_one, zip(srcs, objs)) if e]
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    if force or _stale(LIBRARY, objs):
        tmp = f"{LIBRARY}.{os.getpid()}.tmp"
        r = subprocess.run([exe, *ARCH, "-shared", *objs, "-o", tmp], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"linking {LIBRARY} failed:\n{r.stdout}{r.stderr}")
        os.replace(tmp, LIBRARY)
    return LIBRARY
