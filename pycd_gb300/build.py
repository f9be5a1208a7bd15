"""Build libpycd_gb300.so in-tree with nvcc for sm_103a.

Each .cu file under csrc/ is compiled in parallel to an object, then linked
into ``pycd_gb300/_lib/libpycd_gb300.so``.  A stamp of the sources, the
header and the flags skips the build when nothing changed.
"""
import hashlib
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
OUT_DIR = PKG / "_lib"
LIB = OUT_DIR / "libpycd_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code: no contraction of a*b+c into FMA, so host arithmetic (the exp
# table) gives the same doubles on x86-64 and aarch64 hosts
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-fvisibility=hidden", "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr"]
SOURCES = ["capi.cu", "ewald.cu", "ewald_split.cu", "kmc.cu", "kmc_capped.cu",
           "kmc_cta.cu", "msd.cu"]


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found; the CUDA toolkit is required")
    return cand


def _stamp():
    h = hashlib.sha256()
    for p in sorted(CSRC.glob("*")) + sorted(INCLUDE.glob("*.h")):
        h.update(p.name.encode())
        h.update(p.read_bytes())
    h.update(" ".join(ARCH + NVCC_FLAGS + SOURCES).encode())
    return h.hexdigest()


def build(force=False, verbose=False):
    """Compile (if needed) and return the path of the shared library."""
    OUT_DIR.mkdir(exist_ok=True)
    stamp_file = OUT_DIR / "build.stamp"
    stamp = _stamp()
    if (not force and LIB.exists() and stamp_file.exists()
            and stamp_file.read_text() == stamp):
        return LIB
    nvcc = _nvcc()
    objs = []

    def compile_one(src):
        obj = OUT_DIR / (Path(src).stem + ".o")
        cmd = [nvcc] + ARCH + NVCC_FLAGS + ["-I", str(INCLUDE), "-I", str(CSRC),
                                           "-c", str(CSRC / src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed on %s:\n%s%s" % (src, r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc] + ARCH + ["-shared", "-o", str(tmp)] + [str(o) for o in objs] + [
        "-cudart", "static"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    for o in objs:
        o.unlink(missing_ok=True)
    stamp_file.write_text(stamp)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
