"""Builds libsubwaygb.so (and the drop-in CLI apps) in-tree for sm_103a.

The library is two translation units compiled in parallel: the CUDA engine
(nvcc, one -gencode for sm_103a) and the host graph code (g++ -fopenmp).
Outputs go to subway_gb300/lib/ and subway_gb300/bin/; rebuilding is skipped
when every output is newer than every source.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
LIBDIR = PKG / "lib"
BINDIR = PKG / "bin"
OBJDIR = PKG / "_build"
LIB = LIBDIR / "libsubwaygb.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
APPS = [f"{a}-{m}" for a in ("bfs", "cc", "sssp", "sswp", "pr") for m in ("sync", "async")]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _newer(outputs, inputs) -> bool:
    outs = [Path(o) for o in outputs]
    if not all(o.exists() for o in outs):
        return False
    t_out = min(o.stat().st_mtime for o in outs)
    return all(Path(i).stat().st_mtime <= t_out for i in inputs)


def _run_parallel(cmds, verbose=False):
    procs = []
    for c in cmds:
        if verbose:
            print(" ".join(map(str, c)), flush=True)
        procs.append((c, subprocess.Popen(list(map(str, c)), stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    errors = []
    for c, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            errors.append(f"$ {' '.join(map(str, c))}\n{out.decode(errors='replace')}")
        elif verbose and out:
            print(out.decode(errors="replace"))
    if errors:
        raise RuntimeError("build failed:\n" + "\n".join(errors))


def lib_sources():
    return [CSRC / "sgw_engine.cu", CSRC / "sgw_mlp.cu", CSRC / "sgw_batch.cu", CSRC / "sgw_graph.cpp"]


def lib_deps():
    return lib_sources() + [CSRC / "sgw_kernels.cuh", CSRC / "sgw_internal.h", CSRC / "sgw_mlp.cuh",
                            INCLUDE / "subway_gb300.h", INCLUDE / "sgw_graphgen.h"]


def build_lib(verbose=False, force=False) -> Path:
    if not force and _newer([LIB], lib_deps()):
        return LIB
    LIBDIR.mkdir(exist_ok=True)
    OBJDIR.mkdir(exist_ok=True)
    nv = nvcc()
    cu = [CSRC / "sgw_engine.cu", CSRC / "sgw_mlp.cu", CSRC / "sgw_batch.cu"]
    objs = [OBJDIR / (p.stem + ".o") for p in cu]
    o_cpp = OBJDIR / "sgw_graph.o"
    cmds = [[nv, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
             f"-I{INCLUDE}", "-c", src, "-o", obj] for src, obj in zip(cu, objs)]
    cmds.append(["g++", "-O3", "-std=c++17", "-fPIC", "-fopenmp", f"-I{INCLUDE}",
                 "-c", CSRC / "sgw_graph.cpp", "-o", o_cpp])
    _run_parallel(cmds, verbose)
    tmp = LIB.with_suffix(".so.tmp")
    _run_parallel([[nv, *ARCH, "-shared", *objs, o_cpp, "-o", tmp, "-Xcompiler", "-fopenmp", "-lgomp"]],
                  verbose)
    os.replace(tmp, LIB)
    return LIB


def build_apps(verbose=False, force=False) -> Path:
    src = CSRC / "apps" / "subway_app.cpp"
    hdr = INCLUDE / "subway_gb300.hpp"
    if not src.exists():
        return BINDIR
    BINDIR.mkdir(exist_ok=True)
    main = BINDIR / "subway-app"
    deps = [src, hdr, INCLUDE / "subway_gb300.h", LIB]
    if force or not _newer([main], deps):
        _run_parallel([["g++", "-O2", "-std=c++17", f"-I{INCLUDE}", src, "-o", main,
                        f"-L{LIBDIR}", "-lsubwaygb", f"-Wl,-rpath,{LIBDIR}"]], verbose)
    # one name per reference binary (and tools/converter); the program picks
    # what to do from argv[0]
    for a in APPS + ["converter"]:
        link = BINDIR / a
        if link.is_symlink() or link.exists():
            link.unlink()
        link.symlink_to(main.name)
    return BINDIR


def build(verbose=False, force=False):
    build_lib(verbose, force)
    build_apps(verbose, force)


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
