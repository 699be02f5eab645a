"""Test infrastructure (oracle pinning only): a stand-in for the two pieces of CuPy that the
reference uses, so that its unmodified Python (python/isb_filter.py, python/stitcher.py,
python/depth_estimation.py) runs on CPU tensors.

* ``RawModule(code=...)`` receives the kernel source exactly as the reference assembles it
  (python/vec_utils.cuh + the .cu file, with its macros substituted as text,
  python/isb_filter.py:47-52 and python/stitcher.py:82-93).  The source is piped to ``g++``
  together with oracle/refcuda_shim.h (CUDA built-ins for the host) and the launch harness
  oracle/refcuda_harness_{isb,stitch}.inc, and built into ``oracle/_ref/`` (git-ignored, cached
  by content hash).  The reference source is never written into this repository.
* ``module.get_function(name)(block=..., grid=..., args=...)`` runs the launch through the
  harness: ``data_ptr()`` integers of CPU tensors are host pointers, so the reference kernel
  bodies read and write the torch CPU tensors directly.
* ``float32`` is numpy's float32 (the reference passes scalars as ``cupy.float32``).

This module exists to generate and check golden vectors in a container that has the reference
sources.  The product library never imports it.
"""
from __future__ import annotations

import ctypes
import hashlib
import os
import re
import subprocess

import numpy as np

float32 = np.float32

_HERE = os.path.dirname(os.path.abspath(__file__))
_OUT = os.path.join(_HERE, "_ref")

# argument kinds per reference kernel: p = device pointer, i = int, f = float32
_SIGNATURES = {
    "guideDownsample2xKernel": "ppiippiif",
    "guideUpsample2xKernel": "ppiippiifff",
    "reprojectDistanceKernel": "pppp",
    "createInpaintingWeightsKernel": "ppp",
    "inpaintKernel": "pp",
    "createBlendingLutKernel": "pppppp",
    "mergeRGBDPanoramaKernel": "pppppiipppp",
}
_CTYPES = {"p": ctypes.c_void_p, "i": ctypes.c_int, "f": ctypes.c_float}

CXXFLAGS = ["-std=c++17", "-O2", "-fopenmp", "-fPIC", "-shared", "-fwrapv", "-ffp-contract=off", "-w"]


def build_reference_library(code: str) -> str:
    """Compile reference kernel source text (plus shim and harness) into oracle/_ref; returns the path."""
    kind = "stitch" if "mergeRGBDPanoramaKernel" in code else "isb"
    with open(os.path.join(_HERE, f"refcuda_harness_{kind}.inc")) as f:
        harness = f.read()
    shim = os.path.join(_HERE, "refcuda_shim.h")
    with open(shim) as f:
        shim_text = f.read()
    source = code + "\n" + harness
    defines = []
    if kind == "stitch":
        # COLS * ROWS as substituted into the bounds test of reprojectDistanceKernel (stitcher.cu:186)
        m = re.search(r"reprojectDistanceKernel.*?indexIn\s*<\s*(\d+)\s*\*\s*(\d+)", code, re.S)
        if m is None:
            raise RuntimeError("cannot find the matching resolution in the stitcher source")
        defines = [f"-DREFCUDA_COLS={m.group(1)}", f"-DREFCUDA_ROWS={m.group(2)}"]
    key = hashlib.sha1((source + shim_text + " ".join(CXXFLAGS + defines)).encode()).hexdigest()[:16]
    os.makedirs(_OUT, exist_ok=True)
    path = os.path.join(_OUT, f"refcuda_{kind}_{key}.so")
    if not os.path.exists(path):
        tmp = path + f".{os.getpid()}.tmp"
        cmd = ["g++", *CXXFLAGS, *defines, "-include", shim, "-x", "c++", "-", "-o", tmp]
        subprocess.run(cmd, input=source.encode(), check=True)
        os.replace(tmp, path)
    return path


class _Kernel:
    def __init__(self, lib: ctypes.CDLL, name: str):
        self._fn = getattr(lib, "refcuda_" + name)
        self._kinds = _SIGNATURES[name]
        self._fn.argtypes = [ctypes.c_long, ctypes.c_long] + [_CTYPES[k] for k in self._kinds]
        self._fn.restype = None

    def __call__(self, block, grid, args):
        if len(args) != len(self._kinds):
            raise TypeError(f"expected {len(self._kinds)} kernel arguments, got {len(args)}")
        conv = []
        for kind, a in zip(self._kinds, args):
            if kind == "p":
                conv.append(ctypes.c_void_p(int(a)))
            elif kind == "i":
                conv.append(int(a))
            else:
                conv.append(float(np.float32(a)))
        self._fn(int(grid[0]), int(block[0]), *conv)


class RawModule:
    def __init__(self, code: str):
        self._lib = ctypes.CDLL(build_reference_library(code))

    def get_function(self, name: str) -> _Kernel:
        return _Kernel(self._lib, name)
