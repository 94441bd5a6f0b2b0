"""Compile the reference's own sources in place into ``oracle/_ref/``.

TEST INFRASTRUCTURE ONLY.  The result, ``oracle/_ref/ref_harness``, runs the
reference's host set-up and CPU scheme functions (to pin the oracle) and, on a
GPU machine, the whole reference program (to compare against its GPU kernels).

The reference is compiled from its files as they are, with three build-level
accommodations and no edit to any source line:

* ``gpu_solver.cu:1036-1039`` hold GBK-encoded string literals in a dead
  debug kernel; nvcc's front end rejects them.  The recipe replays nvcc's own
  compilation steps (``nvcc --dryrun``) and, after each preprocessing step,
  re-encodes the preprocessed text from GBK to UTF-8 -- the same effect as a
  ``-finput-charset=GBK`` option, which nvcc lacks.
* ``cudaThreadSynchronize`` (removed from CUDA) is mapped to
  ``cudaDeviceSynchronize`` by the force-included ``oracle/ref_shim.h``,
  which also guards the reference's mis-sized cudaMemcpy calls.
* ``cuPrintf.cu:89`` includes ``sm_11_atomic_functions.h``, which CUDA 13 no
  longer ships; an empty stand-in header is generated under ``_ref/shim``.

``gpu_fvm.cu``'s ``main`` is renamed ``ref_main`` with ``-Dmain=ref_main`` so
the harness can call the whole program.

Sources are taken from the directory named by ``$E2D_REFERENCE`` or, when
that is unset, from a reference checkout beside the repository
(``../reference``); a byte-identical copy is kept under ``_ref/src``
(git-ignored) so that the same recipe can build the harness on a machine
without the checkout.  ``source_dir()`` is the one place that resolves it.
"""
from __future__ import annotations

import os
import shlex
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
REF_FILES = ["gpu_fvm.cuh", "gpu_fvm.cu", "gpu_init.cu", "gpu_solver.cu", "cuPrintf.cu",
             "cuPrintf.cuh"]
# the reference's RAE2822 meshes, staged beside the sources for machines without the checkout
REF_MESHES = ["2822-3k.dat", "2822-1w.dat", "2822-5w.dat"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def checkout_dir() -> str:
    """The reference checkout: ``$E2D_REFERENCE``, else ``../reference``
    beside the repository."""
    return os.environ.get("E2D_REFERENCE") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")


def source_dir() -> str | None:
    """Directory holding the reference sources: the checkout when present
    (staging a copy under ``_ref/src``), else that staged copy, else None."""
    ref = checkout_dir()
    if all(os.path.exists(os.path.join(ref, f)) for f in REF_FILES):
        stage = os.path.join(OUT, "src")
        os.makedirs(stage, exist_ok=True)
        for f in REF_FILES + REF_MESHES:
            dst = os.path.join(stage, f)
            src = os.path.join(ref, f)
            if os.path.exists(src) and (not os.path.exists(dst) or os.path.getmtime(dst) < os.path.getmtime(src)):
                shutil.copyfile(src, dst)
        return ref
    stage = os.path.join(OUT, "src")
    if all(os.path.exists(os.path.join(stage, f)) for f in REF_FILES):
        return stage
    return None


def _transcode(path: str) -> None:
    """Re-encode a preprocessed file line by line: UTF-8 stays, GBK becomes UTF-8."""
    with open(path, "rb") as f:
        raw = f.read().split(b"\n")
    out = []
    for line in raw:
        try:
            line.decode("utf-8")
            out.append(line)
        except UnicodeDecodeError:
            out.append(line.decode("gbk", errors="replace").encode("utf-8"))
    with open(path, "wb") as f:
        f.write(b"\n".join(out))


def _compile(src: str, obj: str, flags: list[str], keep: str) -> None:
    os.makedirs(keep, exist_ok=True)
    cmd = ["nvcc", "--dryrun", "--keep", "--keep-dir", keep, *ARCH, *flags, "-c", src, "-o", obj]
    res = subprocess.run(cmd, capture_output=True, text=True, check=True)
    script = ["set -e"]
    for line in res.stderr.splitlines():
        if not line.startswith("#$ "):
            continue
        body = line[3:]
        name, eq, value = body.partition("=")
        if eq and name.isidentifier() and not body.startswith(("gcc", "\"")):
            body = f"{name}={shlex.quote(value)}"  # nvcc prints these unquoted
        script.append(body)
        toks = shlex.split(body, posix=True) if body.startswith("gcc") else []
        if toks and "-E" in toks and "-o" in toks:
            target = toks[toks.index("-o") + 1]
            script.append(f"{shlex.quote(sys.executable)} -c "
                          f"{shlex.quote('import sys; sys.path.insert(0, %r); import build_ref; build_ref._transcode(sys.argv[1])' % HERE)}"
                          f" {shlex.quote(target)}")
    subprocess.run(["bash", "-c", "\n".join(script)], check=True, cwd=keep)


def build(force: bool = False) -> str | None:
    """Build ``oracle/_ref/ref_harness``; returns its path or None without sources."""
    src_dir = source_dir()
    if src_dir is None:
        return None
    exe = os.path.join(OUT, "ref_harness")
    deps = [os.path.join(src_dir, f) for f in REF_FILES] + [
        os.path.join(HERE, "ref_harness.cu"), os.path.join(HERE, "ref_shim.h"), __file__]
    if not force and os.path.exists(exe) and os.path.getmtime(exe) >= max(map(os.path.getmtime, deps)):
        return exe
    shim = os.path.join(OUT, "shim")
    os.makedirs(shim, exist_ok=True)
    with open(os.path.join(shim, "sm_11_atomic_functions.h"), "w") as f:
        f.write("/* empty stand-in: CUDA 13 no longer ships this header */\n")
    common = ["-O3", f"-I{shim}", "-include", os.path.join(HERE, "ref_shim.h"),
              "-Xcompiler", "-ffp-contract=off", "-w"]
    jobs = {
        "gpu_init.o": (os.path.join(src_dir, "gpu_init.cu"), common),
        "gpu_fvm.o": (os.path.join(src_dir, "gpu_fvm.cu"), common + ["-Dmain=ref_main"]),
        "gpu_solver.o": (os.path.join(src_dir, "gpu_solver.cu"), common),
    }
    keeps = [os.path.join(OUT, "tmp_" + o[:-2]) for o in jobs]
    try:
        with ThreadPoolExecutor(len(jobs)) as ex:
            futs = [ex.submit(_compile, s, os.path.join(OUT, o), fl, k)
                    for (o, (s, fl)), k in zip(jobs.items(), keeps)]
            for fu in futs:
                fu.result()
    finally:
        # nvcc's intermediates (preprocessed text, compiler-written device
        # code) are needed only while the objects are made: none stays behind
        for k in keeps:
            shutil.rmtree(k, ignore_errors=True)
    harness_o = os.path.join(OUT, "ref_harness.o")
    subprocess.run(["nvcc", *ARCH, "-O2", f"-I{src_dir}", "-Xcompiler", "-ffp-contract=off", "-w",
                    "-c", os.path.join(HERE, "ref_harness.cu"), "-o", harness_o], check=True)
    objs = [os.path.join(OUT, o) for o in jobs] + [harness_o]
    subprocess.run(["nvcc", *ARCH, *objs, "-o", exe], check=True)
    return exe


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
