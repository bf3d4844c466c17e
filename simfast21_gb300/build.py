"""Build the CUDA library libsf21hii.so in-tree (sm_103a only).

Each translation unit under csrc/ is compiled by its own nvcc process (in
parallel), then linked into simfast21_gb300/libsf21hii.so.  No cmake, no
torch extension machinery: the product library has plain C entry points
(include/sf21_hii.h).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libsf21hii.so")
DRIVER = os.path.join(HERE, "sf21_hii")
DRIVER_SRC = [os.path.join(HERE, "driver", f) for f in ("sf21_hii_main.c", "sf21_stage.c")]
PK_DRIVER = os.path.join(HERE, "sf21_power3d_f")  # drop-in for tools/power3d_f.c
PK_DRIVER_SRC = [os.path.join(HERE, "driver", "sf21_power3d_main.c")]
T21_DRIVER = os.path.join(HERE, "sf21_t21")  # drop-in for t21.x
T21_DRIVER_SRC = [os.path.join(HERE, "driver", f) for f in ("sf21_t21_main.c", "sf21_stage.c")]
HALO_DRIVER = os.path.join(HERE, "sf21_get_halos")  # drop-in for get_halos.x
HALO_DRIVER_SRC = [os.path.join(HERE, "driver", f) for f in ("sf21_get_halos_main.c", "sf21_stage.c")]
SFR_DRIVER = os.path.join(HERE, "sf21_get_SFR")  # drop-in for get_SFR.x
SFR_DRIVER_SRC = [os.path.join(HERE, "driver", f) for f in ("sf21_get_SFR_main.c", "sf21_stage.c")]
SOURCES = ["kernels_fft.cu", "kernels_plane.cu", "kernels_pipe.cu", "kernels_adj.cu", "kernels_elem.cu",
           "kernels_plain.cu", "kernels_halo.cu", "kernels_cb.cu", "kernels_dt.cu", "kernels_pk.cu", "kernels_t21.cu",
           "kernels_hf.cu", "kernels_sg.cu", "kernels_gen.cu", "kernels_fused.cu", "kernels_gen600.cu", "hii_api.cu", "halo_api.cu", "sfr_api.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found (CUDA toolkit required to build libsf21hii.so)")


def _deps_mtime(roots=None) -> float:
    t = 0.0
    for root in roots or (CSRC, os.path.join(HERE, "..", "include")):
        for f in os.listdir(root):
            if f.endswith((".cu", ".cuh", ".h", ".c")):
                t = max(t, os.path.getmtime(os.path.join(root, f)))
    return t


def _link_exe(exe: str, srcs, force: bool) -> str:
    deps = max(_deps_mtime([os.path.join(HERE, "driver"), os.path.join(HERE, "..", "include")]),
               os.path.getmtime(LIB))
    if not force and os.path.exists(exe) and os.path.getmtime(exe) >= deps:
        return exe
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        raise RuntimeError("no C compiler for the drivers")
    cmd = [cc, "-O2", "-std=c99", "-ffp-contract=off", "-Wall", "-I", os.path.join(HERE, "..", "include"),
           *srcs, "-o", exe + ".tmp", "-L", HERE, "-lsf21hii", "-Wl,-rpath,$ORIGIN", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{os.path.basename(exe)} build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(exe + ".tmp", exe)
    return exe


def build_driver(force: bool = False) -> str:
    """The sf21_hii executable (drop-in for get_HIIbubbles.x), sf21_t21
    (drop-in for t21.x), sf21_get_halos (drop-in for get_halos.x),
    sf21_get_SFR (drop-in for get_SFR.x) and sf21_power3d_f (drop-in for
    tools/power3d_f), linked to the library with an $ORIGIN rpath; returns
    the sf21_hii path."""
    _link_exe(PK_DRIVER, PK_DRIVER_SRC, force)
    _link_exe(T21_DRIVER, T21_DRIVER_SRC, force)
    _link_exe(HALO_DRIVER, HALO_DRIVER_SRC, force)
    _link_exe(SFR_DRIVER, SFR_DRIVER_SRC, force)
    return _link_exe(DRIVER, DRIVER_SRC, force)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile and link libsf21hii.so and the sf21_hii driver; returns the
    library path."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps_mtime():
        build_driver()
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()

    def compile_one(src: str) -> str:
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        cmd = [cc, *ARCH, *NVCC_FLAGS, "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    build_driver(force=True)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
