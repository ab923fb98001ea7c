"""Build the CUDA chemistry library in-tree for sm_103a.

    python -m cmaq_gb300.build

Compiles every translation unit under ``cmaq_gb300/csrc`` (the C ABI, the grid kernels
per mechanism and the generated device code, which is sharded into several files) as
relocatable device code in parallel, then links ``cmaq_gb300/_build/libcmaqchem.so``.
The solver code is compiled with ``-fmad=false``: every fused multiply-add in it is an
explicit ``fma`` so its rounding matches the CPU oracle.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libcmaqchem.so"
# Build variants the autotuner can choose from: name -> (extra nvcc flags of the generated
# mechanism code, extra flags of every translation unit).  The default library caps the
# generated LU / solve / rate / adjoint functions at 80 registers without their L2 prefetch
# of the next rows' workspace (with 24 resident warps per SM the prefetched lines were
# evicted before use: 2.7 % slower, variant pf80), and the work-queue kernel carries launch
# bounds for 24 resident warps per SM; this measured fastest (see the launch-shape sweep in
# profiles/).  The EBI routines and the kernels' own code are not capped.
GEN_DEFAULT = ["-maxrregcount=80"]
Q_DEFAULT = "-DCHEM_QUEUE_WARPS_PER_SM=24"
GEN128 = ["-maxrregcount=128", "-DCHEM_USE_PREFETCH"]
Q8, Q16 = "-DCHEM_QUEUE_WARPS_PER_SM=8", "-DCHEM_QUEUE_WARPS_PER_SM=16"
VARIANTS = {"default": (GEN_DEFAULT, [Q_DEFAULT]),
            "w16": (GEN128, [Q16]),   # 128 registers, 16 warps per SM
            "g168": (["-maxrregcount=168", "-DCHEM_USE_PREFETCH"], []),
            "nopf": (["-maxrregcount=168"], []),
            "full255": ([], [Q8]), "pf255": (["-DCHEM_USE_PREFETCH"], [Q8]),
            "r168": ([], ["-maxrregcount=168"]),
            "r128": ([], ["-maxrregcount=128", Q16]),
            "lucs": ([], ["-DCHEM_LDLU(p)=__ldcs(p)", Q8]),
            # the default build with clock counters between the attempt's phase barriers
            "phases": (GEN_DEFAULT, [Q_DEFAULT, "-DCHEM_PHASE_TIMING"]),
            # 1/U(i,i) by the correctly rounded reciprocal (same bits); L1 prefetch of the next row
            "rcp": (GEN_DEFAULT + ["-DCHEM_RCP(x)=__drcp_rn(x)"], [Q_DEFAULT]),
            "pfl1": (GEN_DEFAULT + ["-DCHEM_USE_PREFETCH_L1"], [Q_DEFAULT]),
            # the default build with the L2 prefetch of the next rows' workspace reads
            "pf80": (["-maxrregcount=80", "-DCHEM_USE_PREFETCH"], [Q_DEFAULT]),
            # other register caps with as many resident warps as they allow
            "r96w20": (["-maxrregcount=96", "-DCHEM_USE_PREFETCH"], ["-DCHEM_QUEUE_WARPS_PER_SM=20"]),
            "r72w28": (["-maxrregcount=72", "-DCHEM_USE_PREFETCH"], ["-DCHEM_QUEUE_WARPS_PER_SM=28"]),
            "r64w32": (["-maxrregcount=64", "-DCHEM_USE_PREFETCH"], ["-DCHEM_QUEUE_WARPS_PER_SM=32"]),
            # KMT2 kernels built for 2 or 3 resident 128-lane blocks per SM (255 / 168 registers;
            # the default is 4, 128 registers), or without the block barriers between phases
            "kq2": (GEN_DEFAULT, [Q_DEFAULT, "-DKMT2_MIN_BLOCKS=2"]),
            "kq3": (GEN_DEFAULT, [Q_DEFAULT, "-DKMT2_MIN_BLOCKS=3"]),
            "kqfree": (GEN_DEFAULT, [Q_DEFAULT, "-DKMT2_LOCKSTEP=0"]),
            # KMT2 refill as soon as a lane is idle, or deferred until 8 or 32 of a block's 128
            # lanes are (the default waits for 16)
            "kqr1": (GEN_DEFAULT, [Q_DEFAULT, "-DKMT2_REFILL_MIN=1"]),
            "kqr8": (GEN_DEFAULT, [Q_DEFAULT, "-DKMT2_REFILL_MIN=8"]),
            "kqr32": (GEN_DEFAULT, [Q_DEFAULT, "-DKMT2_REFILL_MIN=32"])}


def _is_generated_math(src: Path) -> bool:
    """Generated mechanism functions (rates, LU, solves, adjoint, DDM, Gear), not the EBI
    routines: the warp-cooperative EBI kernel is bound by the FP64 pipe, and a 128-register
    cap only added spills (measured 15 % slower)."""
    return src.parent.name == "gen" and not src.name.endswith("_ebi.cu")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-rdc=true", "-fmad=false", "-lineinfo", "-Xcompiler", "-fPIC",
              "-Xptxas", "-O3"]


# The default library's exceptions, measured slower at the 80-register cap: the adjoint's
# own generated routines (called only by the adjoint kernels, launch-bounded for 16 warps
# per SM) and everything of CRACMM2 (twice CB6r5's species: its queue kernel runs 16
# warps per SM with its routines at 128 registers; 56,097 against 51,080 grid-cells/s).
# The KMT2 kernels' own switches (-DKMT2_*) reach kmt2.cu only, so that a KMT2 variant
# shares every other object with the default build.
def _flags(src: Path, variant: str, gen_extra: list, all_extra: list) -> list:
    own = [f for f in all_extra if not f.startswith("-DKMT2_")]
    if src.name != "kmt2.cu":
        all_extra = own
    if variant == "default" or (gen_extra == GEN_DEFAULT and own == [Q_DEFAULT]):
        if src.name.startswith("cracmm2_") or src.name == "mech_cracmm2.cu":
            return [Q16] + (GEN128 if _is_generated_math(src) else [])
        if _is_generated_math(src) and "_adj" in src.name:
            return all_extra + GEN128
    return all_extra + (gen_extra if _is_generated_math(src) else [])


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted((CSRC / "gen").glob("*.cu"))


def _headers() -> list[Path]:
    return (sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted((CSRC / "gen").glob("*.cuh"))
            + sorted((PKG.parent / "include").glob("*.h")))


def lib_path(variant: str = "default") -> Path:
    return LIB if variant == "default" else BUILD / variant / "libcmaqchem.so"


def build(jobs: int | None = None, verbose: bool = False, variant: str = "default") -> Path:
    """Build one variant of ``VARIANTS`` (``default``: generated functions capped at 80
    registers with L2 prefetch, 24 resident warps per SM)."""
    if variant not in VARIANTS:
        raise ValueError(f"unknown variant {variant}")
    out_dir = BUILD if variant == "default" else BUILD / variant
    out_dir.mkdir(parents=True, exist_ok=True)
    import fcntl
    with open(out_dir / ".lock", "w") as lock:      # one builder at a time (ranks of a torchrun job)
        fcntl.flock(lock, fcntl.LOCK_EX)
        return _build_locked(out_dir, variant, jobs, verbose)


def _fresh(obj: Path, src_mtime: float, flags: str) -> bool:
    """obj is newer than its sources and was built with flags."""
    stamp = obj.with_suffix(".flags")
    return obj.exists() and obj.stat().st_mtime > src_mtime and stamp.exists() and stamp.read_text() == flags


def _build_locked(out_dir: Path, variant: str, jobs: int | None, verbose: bool) -> Path:
    lib = lib_path(variant)
    todo_link = False
    gen_extra, all_extra = (list(x) for x in VARIANTS[variant])
    nvcc = _nvcc()
    hdr_mtime = max(p.stat().st_mtime for p in _headers())
    todo, objs = [], []
    for src in sources():
        rel = src.relative_to(CSRC).as_posix().replace("/", "__")
        obj = out_dir / (rel[:-3] + ".o")
        objs.append(obj)
        stamp = obj.with_suffix(".flags")   # the flags the object was built with
        flags = " ".join(_flags(src, variant, gen_extra, all_extra))
        if _fresh(obj, max(src.stat().st_mtime, hdr_mtime), flags):
            continue
        shared = BUILD / obj.name   # the default build's object, when its flags are the same
        if out_dir != BUILD and _fresh(shared, max(src.stat().st_mtime, hdr_mtime), flags):
            shutil.copy2(shared, obj)
            stamp.write_text(flags)
            todo_link = True
            continue
        todo.append((src, obj))

    def compile_one(item):
        src, obj = item
        extra = _flags(src, variant, gen_extra, all_extra)
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, *extra, "-I", str(CSRC), "-c", str(src), "-o", str(obj) + ".tmp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stderr[-4000:]}")
        os.replace(str(obj) + ".tmp", obj)
        obj.with_suffix(".flags").write_text(" ".join(extra))
        if verbose:
            print("compiled", src.name, flush=True)

    if todo:
        with ThreadPoolExecutor(max_workers=jobs or os.cpu_count() or 4) as ex:
            list(ex.map(compile_one, todo))
    if todo or todo_link or not lib.exists():
        cmd = [nvcc, *ARCH, "-shared", "-rdc=true", *[str(o) for o in objs], "-o", str(lib) + ".tmp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr[-4000:]}")
        os.replace(str(lib) + ".tmp", lib)
    return lib


if __name__ == "__main__":
    for v in (sys.argv[1:] or ["default"]):
        print(build(verbose=True, variant=v))
    sys.exit(0)
