"""Build recipe of the GB300 library: every CUDA translation unit compiled for
sm_103a in parallel, linked into ``bio-cfd_gb300/lib/libbiocfd_gb300.so``.

FP64 reference-arithmetic kernels need exact IEEE rounding of every
operation, so device code is compiled with ``--fmad=false`` (kernels that
want fused multiply-adds call ``__fmaf_rn`` / ``fma`` explicitly) and host
code with ``-ffp-contract=off``.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
SRC = PKG / "csrc"
OUT = PKG / "lib" / "libbiocfd_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "-I" + str(ROOT / "include"), "-I" + str(SRC)]


def sources():
    return sorted(SRC.glob("*.cu"))


def build(force: bool = False, verbose: bool = False) -> Path:
    srcs = sources()
    deps = srcs + sorted(SRC.glob("*.h")) + sorted(SRC.glob("*.cuh")) + [ROOT / "include" / "biocfd_gb300.h"]
    if not force and OUT.exists() and all(OUT.stat().st_mtime >= p.stat().st_mtime for p in deps):
        return OUT
    nvcc = os.environ.get("NVCC", "nvcc")
    obj = PKG / "lib" / "obj"
    obj.mkdir(parents=True, exist_ok=True)
    procs = []
    for s in srcs:
        o = obj / (s.stem + ".o")
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-c", str(s), "-o", str(o)]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        procs.append((s, o, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for s, o, p in procs:
        out = p.communicate()[0].decode(errors="replace")
        if p.returncode != 0:
            failed.append((s.name, out))
        elif verbose and out.strip():
            print(f"== {s.name}\n{out}")
    if failed:
        msg = "\n".join(f"---- {n}\n{o}" for n, o in failed)
        raise RuntimeError("nvcc failed:\n" + msg)
    tmp = OUT.with_suffix(".so.tmp%d" % os.getpid())
    subprocess.check_call([nvcc, *ARCH, "-shared", "-o", str(tmp), *[str(o) for _, o, _ in procs]])
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
