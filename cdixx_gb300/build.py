"""Build the CDI path's shared library ``cdixx_gb300/_lib/libcdx.so`` for sm_103a.

Translation units are compiled in parallel with nvcc (one -gencode, no
cmake); the host-only unit with g++.  Incremental: a unit is rebuilt when its
source or any header in ``csrc/`` or ``include/`` is newer than its object.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "_lib"
OBJDIR = LIBDIR / "obj"
LIB = LIBDIR / "libcdx.so"
RUN = LIBDIR / "cdi_run"
GENCODE = "arch=compute_103a,code=sm_103a"

CU_UNITS = ["cdx_api.cu", "cdx_misc.cu", "cdx_dispatch.cu", "cdx_sizes_a.cu", "cdx_sizes_b.cu",
            "cdx_sizes_c.cu", "cdx_sizes_d.cu", "cdx_noalloc.cu", "cdx_unet.cu", "cdx_fwdmodel.cu", "cdx_umma.cu",
            "cdx_ptycho.cu", "cdx_pty_sizes_a.cu", "cdx_pty_sizes_b.cu", "cdx_pty_zernike.cu"]
CC_UNITS = ["cdx_host.cc", "cdx_config.cc", "cdi_shim.cc"]


def _nvcc() -> str:
    n = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(n).exists():
        raise RuntimeError("nvcc not found: the CDI kernels need the CUDA toolkit to build")
    return n


def _headers_mtime() -> float:
    hs = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h*"))
    return max((h.stat().st_mtime for h in hs), default=0.0)


def _compile(cmd, src: Path, obj: Path, hdr_mtime: float) -> str | None:
    if obj.exists() and obj.stat().st_mtime >= max(src.stat().st_mtime, hdr_mtime):
        return None
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return f"{src.name}:\n{r.stdout}\n{r.stderr}"
    return None


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    nvcc = _nvcc()
    OBJDIR.mkdir(parents=True, exist_ok=True)
    hdr = _headers_mtime()
    inc = [f"-I{CSRC}", f"-I{ROOT / 'include'}"]
    tasks = []
    for u in CU_UNITS:
        src, obj = CSRC / u, OBJDIR / (u + ".o")
        cmd = [nvcc, "-std=c++17", "-O3", "-lineinfo", "-gencode", GENCODE, "-Xcompiler", "-fPIC",
               "-Xcompiler", "-fvisibility=hidden", *inc, "-c", str(src), "-o", str(obj)]
        tasks.append((cmd, src, obj))
    for u in CC_UNITS:
        src, obj = CSRC / u, OBJDIR / (u + ".o")
        if not src.exists():
            continue
        cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-fvisibility=hidden", *inc,
               "-I/usr/local/cuda/include", "-c", str(src), "-o", str(obj)]
        tasks.append((cmd, src, obj))
    jobs = jobs or min(len(tasks), os.cpu_count() or 4)
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        errs = [e for e in ex.map(lambda t: _compile(t[0], t[1], t[2], hdr), tasks) if e]
    if errs:
        raise RuntimeError("CUDA build failed:\n" + "\n".join(errs))
    objs = [str(t[2]) for t in tasks]
    newest = max(Path(o).stat().st_mtime for o in objs)
    if not LIB.exists() or LIB.stat().st_mtime < newest:
        cmd = [nvcc, "-shared", "-gencode", GENCODE, "-o", str(LIB) + ".tmp", *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
        os.replace(str(LIB) + ".tmp", LIB)
    # the config-driven driver (the reference's cdi_run), linked against the library
    run_src = CSRC / "cdi_run.cc"
    if not RUN.exists() or RUN.stat().st_mtime < max(LIB.stat().st_mtime, run_src.stat().st_mtime, hdr):
        cmd = ["g++", "-std=c++17", "-O2", *inc, "-I/usr/local/cuda/include", str(run_src), "-o", str(RUN),
               f"-L{LIBDIR}", "-lcdx", "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("cdi_run link failed:\n" + r.stdout + r.stderr)
    # the config-driven ptychography program (the reference's util/ptycho.cpp main)
    pty_src = CSRC / "ptycho_run.cc"
    PTY = LIBDIR / "ptycho_run"
    if not PTY.exists() or PTY.stat().st_mtime < max(LIB.stat().st_mtime, pty_src.stat().st_mtime, hdr):
        cmd = ["g++", "-std=c++17", "-O2", *inc, str(pty_src), "-o", str(PTY), f"-L{LIBDIR}", "-lcdx",
               "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("ptycho_run link failed:\n" + r.stdout + r.stderr)
    # bench-only comparator: the reference's iteration structure on cuFFT (never loaded by the product)
    cmp_src = CSRC / "cufft_cmp.cu"
    CMP = LIBDIR / "libcdx_cufft_cmp.so"
    if not CMP.exists() or CMP.stat().st_mtime < cmp_src.stat().st_mtime:
        cmd = [nvcc, "-std=c++17", "-O3", "-gencode", GENCODE, "-Xcompiler", "-fPIC", "-shared", str(cmp_src), "-o",
               str(CMP) + ".tmp", "-lcufft", "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("comparator build failed:\n" + r.stdout + r.stderr)
        os.replace(str(CMP) + ".tmp", CMP)
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
