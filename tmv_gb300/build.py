"""Build the sm_103a shared library libtmvg.so from tmv_gb300/csrc/*.cu, and
the TMV link-time drop-in (tmv_gb300/shim) where TMV's sources are at hand.

Every CUDA translation unit is compiled by nvcc for sm_103a only, in parallel
and incrementally (an object is rebuilt when its source or any header is
newer), then linked into tmv_gb300/_build/libtmvg.so.  Run as a module or call
build_library().

The drop-in compiles TMV 0.76 itself, so it needs a TMV source tree:
$TMV_REFERENCE when that is set, else the copy that stage_tmv_sources() keeps
in third_party/tmv (git-ignored, never committed: it exists so that TMV can be
compiled on a machine that has no TMV tree of its own).
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = OUT / "libtmvg.so"

THIRD_PARTY_TMV = ROOT / "third_party" / "tmv"
SHIM = PKG / "shim"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
    "-I", str(ROOT / "include"), "-I", str(CSRC),
]


def _nvcc() -> str:
    cand = os.environ.get("NVCC") or "/usr/local/cuda/bin/nvcc"
    return cand if Path(cand).exists() else "nvcc"


def _headers_mtime() -> float:
    hs = list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h"))
    return max((h.stat().st_mtime for h in hs), default=0.0)


def _compile(src: Path, obj: Path, extra: list[str]) -> None:
    cmd = [_nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")


def build_library(verbose: bool = False, extra_flags: list[str] | None = None) -> Path:
    extra = list(extra_flags or [])
    OUT.mkdir(parents=True, exist_ok=True)
    (OUT / "obj").mkdir(exist_ok=True)
    srcs = sorted(CSRC.glob("*.cu"))
    hdr_t = _headers_mtime()
    jobs = []
    objs = []
    for s in srcs:
        o = OUT / "obj" / (s.stem + ".o")
        objs.append(o)
        if not o.exists() or o.stat().st_mtime < max(s.stat().st_mtime, hdr_t):
            jobs.append((s, o))
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            futs = [ex.submit(_compile, s, o, extra) for s, o in jobs]
            for f in futs:
                f.result()
            if verbose:
                print(f"compiled {len(jobs)} translation unit(s)", file=sys.stderr)
    if jobs or not LIB.exists():
        cmd = [_nvcc(), *ARCH, "-shared", "-o", str(LIB), *map(str, objs)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


def _is_tmv_tree(p: Path) -> bool:
    return (p / "src" / "TMV_LUDecompose.cpp").exists() and (p / "include" / "TMV.h").exists()


def tmv_source_dir() -> Path | None:
    """The TMV source tree to compile, or None when there is none."""
    env = os.environ.get("TMV_REFERENCE")
    if env and _is_tmv_tree(Path(env)):
        return Path(env)
    if _is_tmv_tree(THIRD_PARTY_TMV):
        return THIRD_PARTY_TMV
    return None


def stage_tmv_sources(src: str | Path) -> Path:
    """Copy TMV's src/, include/ and licence from `src` to third_party/tmv
    (file times kept, so an unchanged tree rebuilds nothing)."""
    import shutil

    src = Path(src)
    if not _is_tmv_tree(src):
        raise FileNotFoundError(f"{src} is not a TMV source tree")
    THIRD_PARTY_TMV.mkdir(parents=True, exist_ok=True)
    for d in ("src", "include"):
        shutil.copytree(src / d, THIRD_PARTY_TMV / d, dirs_exist_ok=True)
    if (src / "TMV_LICENSE").exists():
        shutil.copy2(src / "TMV_LICENSE", THIRD_PARTY_TMV / "TMV_LICENSE")
    return THIRD_PARTY_TMV


def build_dropin(tmv_src: str | Path, jobs: int | None = None, objects_only: bool = False) -> Path:
    """make -C tmv_gb300/shim: the drop-in, stock TMV and the demo program
    (objects_only: compile TMV and the shim without linking, which needs no
    CUDA library)."""
    if not objects_only:
        build_library()
    jobs = jobs or (os.cpu_count() or 4)
    r = subprocess.run(["make", "-s", f"-j{jobs}", "-C", str(SHIM), f"TMV_SRC={tmv_src}"]
                       + (["objects"] if objects_only else []),
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"drop-in build failed:\n{r.stdout[-4000:]}\n{r.stderr[-4000:]}")
    return SHIM / "_build"


if __name__ == "__main__":
    print(build_library(verbose=True))
