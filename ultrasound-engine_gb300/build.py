"""Build the native parts of usx-gb300 in-tree.

    python ultrasound-engine_gb300/build.py [--no-host] [--no-oracle] [-j N]

Produces
  ultrasound-engine_gb300/lib/libusx_cu.so    CUDA kernels + C-ABI (sm_103a)
  ultrasound-engine_gb300/lib/libusx.so       C++ host API (namespace usx)
  ultrasound-engine_gb300/python/usx/_usx*.so pybind11 module over libusx.so
  oracle/liboracle.so                         CPU oracle (test infrastructure)
  oracle/_ref/libusx_ref.so                   reference build, where its sources exist

Device code is compiled for sm_103a only, with -fmad=false so float
expressions are evaluated exactly as written (see csrc/usx_internal.cuh). Host
code is compiled with -ffp-contract=off for the same reason on aarch64, whose
compilers contract by default.
"""

from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import subprocess
import sys
import sysconfig
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
HOST = PKG / "host"
LIB = PKG / "lib"
PYPKG = PKG / "python" / "usx"
BUILD = PKG / "_build"
INCLUDE = ROOT / "include"
ORACLE = ROOT / "oracle"
CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

CU_SOURCES = ["ctx.cu", "demod.cu", "beamform.cu", "mv_tc.cu", "learned.cu", "mlp.cu", "post.cu", "doppler.cu",
              "simulate.cu", "gemm_tc5.cu"]
FMAD_SOURCES = {"mv_tc.cu", "learned.cu", "mlp.cu", "gemm_tc5.cu"}
HOST_SOURCES = ["types.cpp", "geometry.cpp", "simulator.cpp", "demodulate.cpp", "beamformer.cpp",
                "postprocess.cpp", "doppler.cpp", "pipeline.cpp", "runtime.cpp"]


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps if d.exists())


def _headers() -> list[Path]:
    return [*CSRC.glob("*.cuh"), *INCLUDE.glob("*.h"), *(HOST / "usx").glob("*.hpp")]


def build_cuda(jobs: int) -> Path:
    BUILD.mkdir(exist_ok=True)
    LIB.mkdir(exist_ok=True)
    out = LIB / "libusx_cu.so"
    objs = []
    cmds = []
    for src in CU_SOURCES:
        s = CSRC / src
        o = BUILD / (s.stem + ".o")
        objs.append(o)
        if _stale(o, [s, *_headers()]):
            # Bit-faithful kernels keep every product and sum separately rounded;
            # the tensor-core MV (1e-3 tolerance) contracts freely.
            fmad = "-fmad=true" if src in FMAD_SOURCES else "-fmad=false"
            cmds.append([NVCC, ARCH, "-lineinfo", "-O3", "-std=c++17", fmad,
                         "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
                         "-I", str(INCLUDE), "-c", str(s), "-o", str(o)])
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        list(ex.map(_run, cmds))
    if cmds or _stale(out, objs):
        _run([NVCC, ARCH, "-shared", "-cudart", "shared", "-o", str(out), *map(str, objs),
              "-Xlinker", f"-rpath,{CUDA_HOME / 'lib64'}"])
    return out


def build_host(jobs: int) -> Path:
    """C++ host library (reference-compatible classes) and the _usx module."""
    import torch.utils.cpp_extension as ce  # only for the bundled pybind11 headers

    pyb = [p for p in ce.include_paths() if p.endswith("/include")]
    py_inc = sysconfig.get_paths()["include"]
    cuda_inc = str(CUDA_HOME / "include")
    ext = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    BUILD.mkdir(exist_ok=True)
    common = ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off",
              "-I", str(HOST), "-I", str(INCLUDE), "-I", cuda_inc]
    objs, cmds = [], []
    for src in HOST_SOURCES:
        s = HOST / "src" / src
        o = BUILD / (s.stem + ".host.o")
        objs.append(o)
        if _stale(o, [s, *_headers()]):
            cmds.append(common + ["-c", str(s), "-o", str(o)])
    mod_src = HOST / "pymodule.cpp"
    mod_obj = BUILD / "pymodule.o"
    if _stale(mod_obj, [mod_src, *_headers()]):
        cmds.append(common + ["-fvisibility=hidden", "-I", py_inc, *sum((["-I", p] for p in pyb), []),
                              "-c", str(mod_src), "-o", str(mod_obj)])
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        list(ex.map(_run, cmds))
    libhost = LIB / "libusx.so"
    if cmds or _stale(libhost, objs):
        _run(["g++", "-shared", "-o", str(libhost), *map(str, objs), "-L", str(LIB), "-lusx_cu", "-ldl",
              "-Wl,-rpath,$ORIGIN"])
    for old in PYPKG.glob("_usx*.so"):
        if old.name != "_usx" + ext:
            old.unlink()
    mod = PYPKG / ("_usx" + ext)
    if cmds or _stale(mod, [mod_obj, libhost]):
        _run(["g++", "-shared", "-o", str(mod), str(mod_obj), "-L", str(LIB), "-lusx", "-lusx_cu",
              "-Wl,-rpath,$ORIGIN/../../lib"])
    return mod


def build_oracle() -> Path:
    out = ORACLE / "liboracle.so"
    srcs = [ORACLE / "usx_oracle_f32.c", ORACLE / "usx_oracle_f64.c"]
    if _stale(out, srcs + [ORACLE / "usx_oracle_impl.inc", ORACLE / "usx_oracle.h"]):
        _run(["gcc", "-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-std=c11", "-shared",
              *map(str, srcs), "-o", str(out), "-lm"])
    return out


def build_reference(ref_dir: str | None = None) -> Path | None:
    """The reference engine from its own sources, only where they exist.

    The checkout's location is the recipe's business (oracle/build_ref.sh:
    its argument, else USX_REFERENCE_DIR, else its default); the recipe exits
    with status 3 when there are no sources to build."""
    out = ORACLE / "_ref" / "libusx_ref.so"
    if not _stale(out, [ORACLE / "ref_shim.cpp", ORACLE / "build_ref.sh"]):
        return out
    cmd = ["bash", str(ORACLE / "build_ref.sh")] + ([ref_dir] if ref_dir else [])
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode == 3:
        return None
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return out


def build_all(host: bool = True, oracle: bool = True, jobs: int | None = None) -> None:
    jobs = jobs or max(2, min(8, os.cpu_count() or 2))
    build_cuda(jobs)
    if host:
        build_host(jobs)
    if oracle:
        build_oracle()
        build_reference()


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--no-host", action="store_true")
    ap.add_argument("--no-oracle", action="store_true")
    ap.add_argument("-j", type=int, default=None)
    a = ap.parse_args()
    build_all(host=not a.no_host, oracle=not a.no_oracle, jobs=a.j)
    print("built", LIB)
    return 0


if __name__ == "__main__":
    sys.exit(main())
