"""Build the CPU oracle shared libraries (test infrastructure).

    python oracle/build.py [mech ...]

Compiles ``oracle/ros3_oracle.c`` once per mechanism into
``oracle/_build/liboracle_<mech>.so`` with gcc, and ``oracle/kmt2_oracle.c`` (the
KMT2 aqueous cloud chemistry, one mechanism) into ``oracle/_build/liboracle_kmt2.so``, and
``oracle/hetchem_oracle.c`` (HETCHEM_RATES) once per mechanism into
``oracle/_build/liboracle_hetchem_<mech>.so``.  ``-ffp-contract=off`` keeps the
compiler from fusing operations beyond the explicit ``fma`` calls; no
``-march`` flag, so the library builds the same on x86-64 and aarch64.

The reference's own Fortran (CCTM/src/gas/ros3) cannot be built here: there is no
Fortran compiler, so there is no ``oracle/_ref`` library.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
MECHS = ("cb6r5_ae7_aq", "cracmm2")


def lib_path(mech: str) -> Path:
    return HERE / "_build" / f"liboracle_{mech}.so"


def kmt2_lib_path() -> Path:
    return HERE / "_build" / "liboracle_kmt2.so"


def hetchem_lib_path(mech: str = "cb6r5_ae7_aq") -> Path:
    return HERE / "_build" / f"liboracle_hetchem_{mech}.so"


def _gcc(srcs, out: Path, defines=()):
    return ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
            *defines, "-Wno-unused-function", "-I", str(HERE), *[str(s) for s in srcs], "-o", str(out) + ".tmp", "-lm"]


def build(mechs=MECHS, force: bool = False) -> list[Path]:
    out_dir = HERE / "_build"
    out_dir.mkdir(exist_ok=True)
    src = HERE / "ros3_oracle.c"
    src_ebi = HERE / "ebi_oracle.c"
    procs, outs = [], []
    for mech in mechs:
        gen = HERE / "gen" / f"{mech}_mech.c"
        gen_ebi = HERE / "gen" / f"{mech}_ebi.c"
        out = lib_path(mech)
        outs.append(out)
        newest = max(p.stat().st_mtime for p in (src, src_ebi, gen, gen_ebi, HERE / "oracle.h",
                                                 HERE / "ros3_adjoint.c", HERE / "gear_oracle.c",
                                                 HERE / "portable_pow.h"))
        if not force and out.exists() and out.stat().st_mtime > newest:
            continue
        cmd = _gcc([src, src_ebi], out, (f'-DMECH_SOURCE="gen/{mech}_mech.c"', f'-DEBI_SOURCE="gen/{mech}_ebi.c"'))
        procs.append((subprocess.Popen(cmd, cwd=HERE), out))
    kout = kmt2_lib_path()
    kdeps = (HERE / "kmt2_oracle.c", HERE / "gen" / "kmt2_aq.c", HERE / "gen" / "kmt2_aq_unrolled.c",
             HERE / "portable_pow.h")
    if force or not kout.exists() or kout.stat().st_mtime <= max(p.stat().st_mtime for p in kdeps):
        procs.append((subprocess.Popen(_gcc([kdeps[0]], kout), cwd=HERE), kout))
    for mech in MECHS:
        hout = hetchem_lib_path(mech)
        hdeps = (HERE / "hetchem_oracle.c", HERE / "gen" / f"{mech}_hetchem.h")
        if force or not hout.exists() or hout.stat().st_mtime <= max(p.stat().st_mtime for p in hdeps):
            cmd = _gcc([hdeps[0]], hout, (f'-DHO_TABLES="gen/{mech}_hetchem.h"',))
            procs.append((subprocess.Popen(cmd, cwd=HERE), hout))
    for p, out in procs:
        if p.wait() != 0:
            raise RuntimeError(f"oracle build failed for {out.name}")
        os.replace(str(out) + ".tmp", out)
    return outs


if __name__ == "__main__":
    for p in build(sys.argv[1:] or MECHS, force=True):
        print(p)
