"""Build the native parts of the k-mer graph builder (no cmake, no setuptools).

Outputs, all in this directory (git-ignored):
  libswapgb.so   the C-ABI library (include/swapgb.h): sm_103a kernels + host code
  libswgsynth.so seeded synthetic genome/read generator (tests, benchmarks)
  bin/swap       the `swap -k -c -i -o [-s]` command line
Translation units are compiled in parallel; nvcc targets sm_103a only.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OBJ = PKG / "_build" / "obj"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> Path:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and Path(cand, "bin", "nvcc").exists():
            return Path(cand)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found (set CUDA_HOME)")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n  %s\n%s" % (" ".join(cmd), r.stdout))
    if r.stdout.strip() and os.environ.get("SWG_BUILD_VERBOSE"):
        sys.stderr.write(r.stdout)


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, ptxas_info: bool = False) -> dict[str, Path]:
    cuda = _cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    OBJ.mkdir(parents=True, exist_ok=True)
    (PKG / "bin").mkdir(exist_ok=True)
    headers = [INCLUDE / "swapgb.h", CSRC / "swg_internal.h", CSRC / "dev_util.cuh"]
    common = ["-O3", "-std=c++17", "-I" + str(INCLUDE), "-I" + str(CSRC)]
    jobs = []
    cu = CSRC / "kernels.cu"
    cu_cmd = [nvcc, *ARCH, "-lineinfo", "-Xcompiler", "-fPIC", *common, "-c", str(cu), "-o",
              str(OBJ / "kernels.o")]
    if ptxas_info:
        cu_cmd.insert(1, "-Xptxas=-v")
    jobs.append((OBJ / "kernels.o", [cu, *headers], cu_cmd))
    fr = CSRC / "framing.cu"
    jobs.append((OBJ / "framing.o", [fr, *headers],
                 [nvcc, *ARCH, "-lineinfo", "-Xcompiler", "-fPIC", *common, "-c", str(fr), "-o",
                  str(OBJ / "framing.o")]))
    for name in ("emit.cu", "merge.cu", "prune.cu"):
        src = CSRC / name
        o = OBJ / (name[:-3] + ".o")
        jobs.append((o, [src, CSRC / "text_dev.cuh", *headers],
                     [nvcc, *ARCH, "-lineinfo", "-Xcompiler", "-fPIC", *common, "-c", str(src), "-o",
                      str(o)]))
    na = CSRC / "noalloc.cu"
    jobs.append((OBJ / "noalloc.o", [na, *headers],
                 [nvcc, *ARCH, "-lineinfo", "-Xcompiler", "-fPIC", *common, "-c", str(na), "-o",
                  str(OBJ / "noalloc.o")]))
    for name in ("api.cpp", "reads.cpp", "writers.cpp", "server.cpp", "autotune.cpp"):
        src = CSRC / name
        o = OBJ / (name[:-4] + ".o")
        jobs.append((o, [src, *headers], ["g++", "-fPIC", "-pthread", "-Wall", *common,
                                          "-I" + str(cuda / "include"), "-c", str(src), "-o", str(o)]))
    synth_o = OBJ / "synth.o"
    jobs.append((synth_o, [CSRC / "synth.cpp", CSRC / "synth.h"],
                 ["g++", "-fPIC", "-pthread", "-Wall", "-ffp-contract=off", *common, "-c",
                  str(CSRC / "synth.cpp"), "-o",
                  str(synth_o)]))
    main_o = OBJ / "swap_main.o"
    jobs.append((main_o, [CSRC / "swap_main.cpp", INCLUDE / "swapgb.h"],
                 ["g++", "-Wall", *common, "-c", str(CSRC / "swap_main.cpp"), "-o", str(main_o)]))
    todo = [j for j in jobs if ptxas_info and j[0].name == "kernels.o" or _stale(j[0], j[1])]
    with cf.ThreadPoolExecutor(max_workers=len(todo) or 1) as ex:
        list(ex.map(lambda j: _run(j[2]), todo))

    lib = PKG / "libswapgb.so"
    lib_objs = [OBJ / n for n in ("kernels.o", "framing.o", "emit.o", "merge.o", "prune.o", "noalloc.o", "api.o", "reads.o",
                                  "writers.o", "server.o", "autotune.o")]
    if _stale(lib, lib_objs):
        _run([nvcc, *ARCH, "-shared", "-o", str(lib), *map(str, lib_objs), "-lpthread", "-ldl"])
    synth = PKG / "libswgsynth.so"
    if _stale(synth, [synth_o]):
        _run(["g++", "-shared", "-pthread", "-o", str(synth), str(synth_o)])
    swap = PKG / "bin" / "swap"
    if _stale(swap, [main_o, lib]):
        _run(["g++", "-o", str(swap), str(main_o), "-L" + str(PKG), "-lswapgb",
              "-Wl,-rpath,$ORIGIN/..", "-pthread"])
    if verbose:
        print("built", lib, synth, swap)
    return {"lib": lib, "synth": synth, "swap": swap}


def build_oracle(verbose: bool = False, ref_dir: str | None = None) -> None:
    """CPU restatement (always) and, when ref_dir (else the environment
    variable SWG_REFERENCE_DIR) names the reference's source tree, the
    reference itself (oracle/_ref) — test infrastructure, not the product."""
    oracle = ROOT / "oracle"
    _run(["make", "-s", "-C", str(oracle), "-j4", "restatement"])
    ref = ref_dir or os.environ.get("SWG_REFERENCE_DIR")
    if ref and Path(ref, "graph.cpp").exists():
        _run(["make", "-s", "-C", str(oracle), "-j4", "reference", "REF=" + ref])
    if verbose:
        print("built oracle")


if __name__ == "__main__":
    build(verbose=True, ptxas_info="--ptxas" in sys.argv)
    build_oracle(verbose=True)
