"""Build ``libeuler2d.so`` (and the ``e2d_solve`` command) for sm_103a in-tree.

nvcc cross-compiles without a GPU, so this runs on any machine with the CUDA
13 toolkit.  Translation units are compiled in parallel.  Both stencil
precisions are compiled without multiply-add contraction (``--fmad=false``):
the FP64 kernels so that they reproduce the CPU oracle bit for bit, the FP32
kernels so that every inlined copy of a device function rounds alike (their
fused multiply-adds are explicit ``fmaf`` calls); the FP32 kernels use fast
division / square root and flush denormals.
Host code is compiled with ``-ffp-contract=off`` so the set-up geometry is the
same IEEE arithmetic on x86-64 and aarch64.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "lib")
OBJDIR = os.path.join(PKG, "_build")
LIB = os.path.join(LIBDIR, "libeuler2d.so")
CLI = os.path.join(LIBDIR, "e2d_solve")
COMPAT = os.path.join(LIBDIR, "libeuler2d_compat.a")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = [*ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
               "-Xcompiler", "-ffp-contract=off", f"-I{os.path.join(ROOT, 'include')}"]

GXX = ["g++", "-O2", "-fPIC", "-std=c++17", "-ffp-contract=off", "-Wall",
       f"-I{os.path.join(ROOT, 'include')}"]
UNITS = {
    "mesh.o": ("mesh.cpp", GXX),
    "output.o": ("output.cpp", GXX),
    "solver.o": ("solver.cu", ["nvcc", *NVCC_COMMON]),
    "batch.o": ("batch.cu", ["nvcc", *NVCC_COMMON]),
    "mlp.o": ("mlp.cu", ["nvcc", *NVCC_COMMON]),
    "resid.o": ("resid.cu", ["nvcc", *NVCC_COMMON]),
    "integrals.o": ("integrals.cu", ["nvcc", *NVCC_COMMON]),  # host code only
    "kernels_f64.o": ("kernels_f64.cu", ["nvcc", *NVCC_COMMON, "--fmad=false"]),
    "noalloc.o": ("noalloc.cu", ["nvcc", *NVCC_COMMON, "--fmad=false"]),
    # FP32 stencil: no multiply-add contraction either, so every inlined copy
    # of a device function (single-case and batched kernels, both cells of a
    # face) rounds the same way and gives the same bits
    "kernels_f32.o": ("kernels_f32.cu", ["nvcc", *NVCC_COMMON,
                                          f"--fmad={os.environ.get('E2D_FP32_FMAD', 'false')}",
                                          "-prec-div=false", "-prec-sqrt=false", "-ftz=true"]),
}
HEADERS = ["internal.h", "dev_types.h", "kernels.cuh", "pdl.cuh", "solver_internal.h", "mlp_kernels.cuh", "mlp_tma.cuh"]


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(obj: str, src: str, cmd: list[str], verbose_ptxas: bool) -> None:
    extra = ["-Xptxas", "-v"] if verbose_ptxas and cmd[0] == "nvcc" else []
    if cmd[0] == "nvcc":  # tuning experiments: extra nvcc flags, e.g. -DE2D_MINB_FACES=6
        extra += os.environ.get("E2D_NVCC_EXTRA", "").split()
    full = [*cmd, *extra, "-c", os.path.join(CSRC, src), "-o", os.path.join(OBJDIR, obj)]
    res = subprocess.run(full, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(full)}\n{res.stdout}\n{res.stderr}")
    if verbose_ptxas:
        sys.stderr.write(res.stderr)


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(OBJDIR, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "euler2d.h"),
                                                       __file__]
    # rebuild everything when the extra nvcc flags differ from the last build
    stamp = os.path.join(OBJDIR, "nvcc_extra.txt")
    extra = os.environ.get("E2D_NVCC_EXTRA", "") + "|fp32_fmad=" + os.environ.get("E2D_FP32_FMAD", "false")
    if not os.path.exists(stamp) or open(stamp).read() != extra:
        force = True
        with open(stamp, "w") as f:
            f.write(extra)
    todo = []
    for obj, (src, cmd) in UNITS.items():
        deps = [os.path.join(CSRC, src), *hdrs]
        if force or verbose_ptxas or _stale(os.path.join(OBJDIR, obj), deps):
            todo.append((obj, src, cmd))
    with ThreadPoolExecutor(max(1, len(todo))) as ex:
        for f in [ex.submit(_compile, o, s, c, verbose_ptxas) for o, s, c in todo]:
            f.result()
    objs = [os.path.join(OBJDIR, o) for o in UNITS]
    if force or todo or _stale(LIB, objs):
        tmp = LIB + ".tmp"
        subprocess.run(["nvcc", *ARCH, "-shared", "-o", tmp, *objs], check=True)
        os.replace(tmp, LIB)
    cli_src = os.path.join(CSRC, "e2d_solve_main.cpp")
    if force or _stale(CLI, [cli_src, LIB]):
        subprocess.run(["g++", "-O2", "-std=c++17", f"-I{os.path.join(ROOT, 'include')}", cli_src,
                        "-o", CLI, f"-L{LIBDIR}", "-leuler2d", "-Wl,-rpath,$ORIGIN"], check=True)
    # the reference's function surface, for linking the reference's gpu_fvm.cu
    compat_src = os.path.join(CSRC, "compat.cpp")
    compat_o = os.path.join(OBJDIR, "compat.o")
    compat_deps = [compat_src, os.path.join(ROOT, "include", "euler2d_compat.h"), *hdrs]
    if force or _stale(COMPAT, compat_deps):
        subprocess.run([*GXX, "-I/usr/local/cuda/include", "-c", compat_src, "-o", compat_o], check=True)
        if os.path.exists(COMPAT):
            os.remove(COMPAT)
        subprocess.run(["ar", "rcs", COMPAT, compat_o], check=True)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="--ptxas" in sys.argv))
