"""Host (CPU) build of the CUDA kernels' column routines, for tests.

``lib()`` compiles ``tests/emul/emul.cu`` with nvcc as host code
(``-ffp-contract=off``; glibc math) into ``tests/emul/_build/libxc_emul.so``.
"""
import ctypes
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "_build", "libxc_emul.so")
_lib = None


def _sources():
    csrc = os.path.join(ROOT, "xcape_gb300", "csrc")
    return [os.path.join(HERE, "emul.cu")] + [os.path.join(csrc, f) for f in os.listdir(csrc)
                                              if f.endswith((".cuh", ".h"))]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    return None


def lib():
    global _lib
    if _lib is None:
        stale = not os.path.exists(OUT) or any(os.path.getmtime(s) > os.path.getmtime(OUT)
                                               for s in _sources())
        if stale:
            os.makedirs(os.path.dirname(OUT), exist_ok=True)
            subprocess.run([nvcc(), "-O2", "-std=c++17", "--expt-relaxed-constexpr", "-shared",
                            "-Xcompiler", "-fPIC,-ffp-contract=off", "-o", OUT,
                            os.path.join(HERE, "emul.cu")], check=True)
        L = ctypes.CDLL(OUT)
        vp, i, f, d, ll = (ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_double,
                           ctypes.c_longlong)
        L.emu_cape.argtypes = [i] + [vp] * 6 + [i, f, i, f, i, vp, i, ll] + [vp] * 6 + [i, vp, vp]
        L.emu_cape64.argtypes = [i] + [vp] * 6 + [i, f, i, f, i, vp, i, ll] + [vp] * 5
        L.emu_guess_eval.argtypes = [vp, f, f, f]
        L.emu_guess_eval.restype = f
        L.emu_guess_eval_packed.argtypes = [vp, f, f, f]
        L.emu_guess_eval_packed.restype = f
        L.emu_guess_pairs.argtypes = [ll, ctypes.c_ulonglong, vp, vp, vp, vp]
        L.emu_accel_map.argtypes = [i] + [f] * 10 + [vp]
        L.emu_accel_map.restype = f
        L.emu_request_layout.argtypes = [vp]
        L.emu_srh.argtypes = [i] + [vp] * 10 + [i, vp, d, d, i, ll] + [vp] * 5 + [i]
        L.emu_pres_lev_pos.argtypes = [vp, vp, i, i, ll, vp]
        _lib = L
    return _lib
