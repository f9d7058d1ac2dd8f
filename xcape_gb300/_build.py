"""Build libxcape_gb300.so in-tree with nvcc for sm_103a.

The translation units under ``xcape_gb300/csrc`` are compiled in parallel
(``-gencode arch=compute_103a,code=sm_103a -lineinfo -O3``) and linked into
``xcape_gb300/lib/libxcape_gb300.so``.  Rebuilds only when a source is newer
than the library.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libxcape_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
              "-Xcompiler", "-fPIC", "-I", INCLUDE]

SOURCES = ["capi.cu", "cape_kernel.cu", "srh_kernel.cu", "noalloc.cu", "guess_mlp.cu", "batch.cu",
           "cape_diag.cu", "cape_srh.cu", "pipe_peaks.cu", "cape_retry.cu",
           "srh_seg.cu"]

# Per-file flags.  The SRH path is FP64 hypsometry feeding FP32 Bunkers
# arithmetic whose reference goldens are pinned to 1e-5: it is built without
# FMA contraction so that every float operation rounds as the Fortran's does.
# XC_CAPE_FMAD=0 builds the CAPE kernels the same way (a measurement switch).
def _file_flags(src):
    if src == "srh_kernel.cu":
        return ["-fmad=false"]
    if src == "cape_kernel.cu" and os.environ.get("XC_CAPE_FMAD", "1") == "0":
        return ["-fmad=false"]
    return []


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build xcape_gb300")


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(INCLUDE, "xcape_gb300.h"))
    files.append(os.path.abspath(__file__))
    return files


def needs_build():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(f) > t for f in _deps())


def build(force=False, verbose=False, ptxas_info=False):
    if not force and not needs_build():
        return LIB
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    procs = []
    objs = []
    for src in SOURCES:
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(obj)
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, *_file_flags(src), *extra, "-c",
               os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    errors = []
    for src, p in procs:
        out, _ = p.communicate()
        text = out.decode(errors="replace")
        if p.returncode != 0:
            errors.append(f"--- {src} ---\n{text}")
        elif verbose or ptxas_info:
            print(text, file=sys.stderr)
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    tmp = LIB + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout.decode(errors="replace"))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
