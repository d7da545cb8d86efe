"""Build recipe for the CPU oracle (test infrastructure only).

Compiles the FP64 restatement in this directory into
``oracle/build/liborc.so`` with ``-ffp-contract=off`` so that every
expression rounds exactly as written (no fused multiply-adds), which is the
arithmetic of the reference's serial CPU build.  Loops whose result does not
depend on their order run under OpenMP; the results equal the serial ones.

The reference itself (Fortran 2008 + OpenACC) cannot be compiled in this
environment -- no Fortran compiler exists on either machine -- so there is
no ``oracle/_ref`` build.

``dual=K`` builds the same sources with ``-DORC_DUAL=K`` into
``oracle/build/liborc_dual.so``: every floating-point value is a forward-mode
dual number with K tangent lanes (``orc_real.h``), which makes the oracle an
FP64 tangent-linear model of the whole time step whose value part is bit for
bit the double build's.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
DUAL_LANES = 6
SOURCES = ["orc_navier.cpp", "orc_forcing.cpp", "orc_pcor.cpp", "orc_search.cpp",
           "orc_interp.cpp", "orc_stress.cpp", "orc_motion.cpp", "orc_blockmove.cpp", "orc_api.cpp"]


def lib_path(checked: bool = True, dual: bool = False) -> Path:
    if dual:
        return HERE / "build" / "liborc_dual.so"
    return HERE / "build" / ("liborc.so" if checked else "liborc_fast.so")


def build(checked: bool = True, force: bool = False, dual: bool = False) -> Path:
    """Compile the oracle; ``checked`` keeps the 1-based bounds checks;
    ``dual`` gives the tangent-linear build (DUAL_LANES lanes, checked)."""
    out = lib_path(checked, dual)
    srcs = [HERE / s for s in SOURCES] + [HERE / "orc_core.h", HERE / "orc_real.h"]
    if not force and out.exists() and all(out.stat().st_mtime >= s.stat().st_mtime for s in srcs):
        return out
    out.parent.mkdir(parents=True, exist_ok=True)
    objdir = out.parent / ("obj_dual" if dual else "obj" if checked else "obj_fast")
    objdir.mkdir(exist_ok=True)
    # OpenMP: the order-independent loops (sweeps of one colour, per-cell
    # stencils without thin-surface cells, per-cell searches, maxima) run on
    # all host cores with the serial loops' results
    flags = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall", "-fopenmp"]
    if not checked and not dual:
        flags.append("-DORC_NOCHECK")
    if dual:
        flags.append("-DORC_DUAL=%d" % DUAL_LANES)
    procs, objs = [], []
    for s in SOURCES:
        o = objdir / (Path(s).stem + ".o")
        objs.append(o)
        procs.append(subprocess.Popen(["g++", *flags, "-c", str(HERE / s), "-o", str(o)]))
    if any(p.wait() != 0 for p in procs):
        raise RuntimeError("oracle compile failed")
    tmp = out.with_suffix(".so.tmp%d" % os.getpid())
    subprocess.check_call(["g++", "-shared", "-fopenmp", "-o", str(tmp), *map(str, objs)])
    os.replace(tmp, out)
    return out


if __name__ == "__main__":
    print(build(checked="--fast" not in sys.argv, force="--force" in sys.argv, dual="--dual" in sys.argv))
