"""Build libtridiag.so (and the `test` driver) in-tree with nvcc for sm_103a.

    python -m tridiagonalsolver_gb300.build [--force] [--jobs N]

Objects go to tridiagonalsolver_gb300/lib/obj/, the library and the driver
to tridiagonalsolver_gb300/lib/ (git-ignored).  Each .cu/.cpp under csrc/
is one translation unit compiled in parallel; a unit is rebuilt when it or
any header in csrc/ or include/ is newer than its object.
"""
from __future__ import annotations

import argparse
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
LIB_DIR = PKG / "lib"
OBJ_DIR = LIB_DIR / "obj"
LIB = LIB_DIR / "libtridiag.so"
DRIVER = LIB_DIR / "test"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xptxas", "-warn-spills", "-I", str(INCLUDE)]
LINK_LIBS = ["-lcusparse"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _headers() -> list[Path]:
    return sorted(list(CSRC.rglob("*.cuh")) + list(CSRC.rglob("*.h")) + list(INCLUDE.glob("*.h")))


def _stale(src: Path, obj: Path, deps: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return src.stat().st_mtime > t or any(h.stat().st_mtime > t for h in deps)


def _compile(src: Path, obj: Path, verbose: bool) -> tuple[Path, int, str]:
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
    if src.suffix == ".cpp":
        cmd = [nvcc(), "-x", "c++", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I", str(INCLUDE),
               "-c", str(src), "-o", str(obj)]
    if verbose:
        print(" ".join(cmd), flush=True)
    p = subprocess.run(cmd, capture_output=True, text=True)
    return src, p.returncode, p.stdout + p.stderr


def build(force: bool = False, jobs: int | None = None, verbose: bool = False) -> Path:
    OBJ_DIR.mkdir(parents=True, exist_ok=True)
    deps = _headers()
    lib_srcs = sorted(p for p in CSRC.glob("*.cu"))
    work = []
    objs = []
    for src in lib_srcs:
        obj = OBJ_DIR / (src.stem + ".o")
        objs.append(obj)
        if force or _stale(src, obj, deps):
            work.append((src, obj))
    jobs = jobs or min(len(work) or 1, os.cpu_count() or 4)
    if work:
        with ThreadPoolExecutor(max_workers=jobs) as ex:
            results = list(ex.map(lambda sw: _compile(sw[0], sw[1], verbose), work))
        failed = [(s, out) for s, rc, out in results if rc != 0]
        for s, rc, out in results:
            if out.strip() and (verbose or rc != 0 or "spill" in out or "warning" in out.lower()):
                print(f"--- {s.name}\n{out}", file=sys.stderr)
        if failed:
            raise RuntimeError("nvcc failed for: " + ", ".join(s.name for s, _ in failed))
    if force or work or not LIB.exists():
        cmd = [nvcc(), *ARCH, "-shared", "-cudart", "shared", "-o", str(LIB), *map(str, objs), *LINK_LIBS]
        if verbose:
            print(" ".join(cmd), flush=True)
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("link failed:\n" + p.stdout + p.stderr)
    drv_src = CSRC / "driver" / "test.cpp"
    if drv_src.exists() and (force or not DRIVER.exists() or DRIVER.stat().st_mtime < max(
            [LIB.stat().st_mtime, drv_src.stat().st_mtime] + [h.stat().st_mtime for h in deps])):
        cmd = [nvcc(), "-x", "c++", "-O2", "-std=c++17", "-I", str(INCLUDE), str(drv_src), "-o", str(DRIVER),
               "-L", str(LIB_DIR), "-ltridiag", "-cudart", "shared", f"-Xlinker=-rpath,$ORIGIN"]
        if verbose:
            print(" ".join(cmd), flush=True)
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("driver build failed:\n" + p.stdout + p.stderr)
    return LIB


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--jobs", type=int, default=None)
    ap.add_argument("-v", "--verbose", action="store_true")
    args = ap.parse_args()
    print(build(force=args.force, jobs=args.jobs, verbose=args.verbose))


if __name__ == "__main__":
    main()
