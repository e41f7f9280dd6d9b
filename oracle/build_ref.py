"""Builds the Subway reference (the upstream CUDA/C++ sources) for sm_103a.

TEST AND BASELINE INFRASTRUCTURE.  Outputs only under oracle/_ref/ (git-ignored):

  oracle/_ref/src/        the reference's shared/ and subway/ sources, copied
                          verbatim from the reference tree when it is present
                          (SUBWAY_REFERENCE_TREE), so that a GPU machine
                          without the reference tree can compile them too
  oracle/_ref/bin/        the ten apps as shipped (bfs-sync ... pr-async)
  oracle/_ref/bin_fixed/  the same apps with the host-gather chunk size
                          rounded up (shared/subgraph_generator.cu:75 divides
                          before ceil(), so the last numActive % 64 vertices
                          keep stale edges when numActive >= 50000)

The reference's own Makefiles are not used: its flags (-arch=sm_60,
-std=c++11) do not build with CUDA 13.  Every translation unit is compiled
directly with nvcc -std=c++17 for sm_103a, in parallel.  shared/subgraph.cu is
compiled with -include oracle/ref_budget.h so that SUBWAY_BUDGET_BYTES caps the
device memory the reference sizes its edge buffer from.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
# Where the upstream Subway tree is read from when it is present (the build
# container mounts it there); elsewhere the copy staged under oracle/_ref/src
# is compiled.
REF_TREE = Path(os.environ.get("SUBWAY_REFERENCE_TREE", "/root/reference"))
OUT = HERE / "_ref"
SRC = OUT / "src"
OBJ = OUT / "obj"
APPS = [f"{a}-{m}" for a in ("bfs", "cc", "sssp", "sswp", "pr") for m in ("sync", "async")]
SHARED_CU = ["argument_parsing", "graph", "subgraph", "partitioner", "subgraph_generator", "gpu_kernels", "test"]
SHARED_CPP = ["timer", "subway_utilities"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
B2_OLD = "unsigned int chunkSize = ceil(numActiveNodes / numThreads);"
B2_NEW = "unsigned int chunkSize = (numActiveNodes + numThreads - 1) / numThreads;"


def stage() -> bool:
    """Copies the reference sources into oracle/_ref/src when the tree exists."""
    if not REF_TREE.exists():
        return (SRC / "shared" / "graph.cu").exists()
    for sub in ("shared", "subway"):
        (SRC / sub).mkdir(parents=True, exist_ok=True)
        for f in (REF_TREE / sub).iterdir():
            if f.suffix in (".cu", ".cuh", ".hpp", ".cpp", ".h"):
                dst = SRC / sub / f.name
                if not dst.exists() or dst.read_bytes() != f.read_bytes():
                    shutil.copyfile(f, dst)
    # the B2-fixed variant of the generator
    gen = (SRC / "shared" / "subgraph_generator.cu").read_text()
    if gen.count(B2_OLD) != 1:
        raise RuntimeError("unexpected subgraph_generator.cu: cannot derive the fixed variant")
    fixed = SRC / "shared" / "subgraph_generator_fixed.cu"
    txt = gen.replace(B2_OLD, B2_NEW)
    if not fixed.exists() or fixed.read_text() != txt:
        fixed.write_text(txt)
    return True


def _nvcc():
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def _stale(out: Path, deps) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build_ref(verbose: bool = False) -> bool:
    """Compiles both variants; returns False when no sources are available."""
    if not stage():
        return False
    nv = _nvcc()
    OBJ.mkdir(parents=True, exist_ok=True)
    sh = SRC / "shared"
    headers = list(sh.glob("*.cuh")) + list(sh.glob("*.hpp"))
    jobs = []
    objs = {}
    for name in SHARED_CU + ["subgraph_generator_fixed"]:
        src = sh / f"{name}.cu"
        obj = OBJ / f"{name}.o"
        objs[name] = obj
        extra = ["-include", str(HERE / "ref_budget.h")] if name == "subgraph" else []
        if _stale(obj, [src, HERE / "ref_budget.h", *headers]):
            jobs.append([nv, *ARCH, "-O3", "-std=c++17", "-w", *extra, "-c", str(src), "-o", str(obj)])
    for name in SHARED_CPP:
        src = sh / f"{name}.cpp"
        obj = OBJ / f"{name}.o"
        objs[name] = obj
        if _stale(obj, [src, *headers]):
            jobs.append(["g++", "-O3", "-std=c++17", "-w", "-c", str(src), "-o", str(obj)])
    for app in APPS:
        src = SRC / "subway" / f"{app}.cu"
        obj = OBJ / f"app-{app}.o"
        objs["app-" + app] = obj
        if _stale(obj, [src, *headers]):
            jobs.append([nv, *ARCH, "-O3", "-std=c++17", "-w", "-c", str(src), "-o", str(obj)])
    _parallel(jobs, verbose)
    links = []
    for variant, gen in (("bin", "subgraph_generator"), ("bin_fixed", "subgraph_generator_fixed")):
        (OUT / variant).mkdir(exist_ok=True)
        deps = [objs[n] for n in SHARED_CU if n != "subgraph_generator"] + [objs[gen]] + \
               [objs[n] for n in SHARED_CPP]
        for app in APPS:
            exe = OUT / variant / app
            if _stale(exe, deps + [objs["app-" + app]]):
                links.append([nv, *ARCH, str(objs["app-" + app]), *map(str, deps), "-o", str(exe)])
    _parallel(links, verbose)
    return True


def _parallel(cmds, verbose):
    procs = []
    for c in cmds:
        if verbose:
            print(" ".join(c), flush=True)
        procs.append((c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    bad = []
    for c, p in procs:
        out, _ = p.communicate()
        if p.returncode:
            bad.append(" ".join(c) + "\n" + out.decode(errors="replace"))
    if bad:
        raise RuntimeError("reference build failed:\n" + "\n".join(bad))


def binary(app: str, fixed: bool = False) -> Path:
    return OUT / ("bin_fixed" if fixed else "bin") / app


if __name__ == "__main__":
    ok = build_ref(verbose="-v" in sys.argv)
    print("built" if ok else "no reference sources")
