"""Build the sm_103a library and the host-side element check, in tree.

    python -m nalu_gb300.build            # library + host check
Outputs:
    nalu_gb300/_lib/libnalu_gb300.so      (CUDA kernels + C ABI)
    nalu_gb300/_lib/libnalu_elemcheck.so  (element math compiled for the host)
Each .cu file compiles in its own nvcc process, in parallel, for
-gencode arch=compute_103a,code=sm_103a only.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
SOURCES = ["api.cu", "assemble.cu", "assemble_df.cu", "assemble_df_sd.cu", "assemble_df_c0.cu", "assemble_df_c1.cu",
           "assemble_df_c2.cu", "assemble_ip8_c0.cu", "assemble_ip8_c12.cu", "assemble_ip8_sd.cu", "assemble_ip16_c0.cu",
           "assemble_ip16_c12.cu", "assemble_ip16_sd.cu", "momentum.cu", "momentum_df.cu", "krylov.cu", "cg_fast.cu", "batch.cu", "learned.cu", "train_tc.cu", "multilevel.cu", "geometry.cu", "mass.cu", "faces.cu", "dump.cu", "master_element.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), p.stdout, p.stderr))
    return p.stdout + p.stderr


def build(verbose=False, ptxas_info=False):
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    objs = []
    flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
                    "-I" + CSRC]
    if ptxas_info:
        flags += ["-Xptxas", "-v"]
    # extra compile definitions, e.g. NALU_NVCC_DEFINES="NALU_DF_MINB=6"
    flags += ["-D" + d for d in os.environ.get("NALU_NVCC_DEFINES", "").split() if d]

    def comp(src):
        obj = os.path.join(OUT, src.replace(".cu", ".o"))
        log = _run([nvcc] + flags + ["-c", os.path.join(CSRC, src), "-o", obj])
        return obj, log

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        for obj, log in ex.map(comp, SOURCES):
            objs.append(obj)
            if verbose and log.strip():
                print(log)
    lib = os.path.join(OUT, "libnalu_gb300.so")
    _run([nvcc] + ARCH + ["-shared", "-o", lib] + objs + ["-lcudart"])
    check = os.path.join(OUT, "libnalu_elemcheck.so")
    cxx = shutil.which("g++") or "g++"
    # -ffp-contract=off: the double-float sequences must not be fused
    _run([cxx, "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-shared", "-o", check,
          os.path.join(CSRC, "elem_hostcheck.cpp")])
    # C++ callers of the host interface (include/nalu_gb300.hpp)
    for ex in ("heat_conduction", "continuity_step"):
        _run([cxx, "-std=c++17", "-O2", "-o", os.path.join(OUT, ex), os.path.join(HERE, "examples", ex + ".cpp"),
              "-L" + OUT, "-lnalu_gb300", "-Wl,-rpath," + OUT])
    for o in objs:
        os.remove(o)
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv))
