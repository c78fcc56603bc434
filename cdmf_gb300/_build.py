"""In-tree build of the native parts: libcdmf_cuda.so (CUDA engine + host
helpers, sm_103a only) and the `cdmf` command-line driver.

Plain nvcc/g++ invocations, translation units compiled in parallel; outputs
land in cdmf_gb300/lib and cdmf_gb300/bin (git-ignored).
"""
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INC = os.path.join(ROOT, "include")
LIBDIR = os.path.join(PKG, "lib")
BINDIR = os.path.join(PKG, "bin")
OBJDIR = os.path.join(ROOT, "_build")
LIB = os.path.join(LIBDIR, "libcdmf_cuda.so")
CLI = os.path.join(BINDIR, "cdmf")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-fopenmp", "-I", INC]
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-I", INC]

CU_SOURCES = ["engine.cu", "noalloc.cu", "compress.cu"]
# launch.cu holds the kernel launchers; it is compiled once per residual type
# (0 = FP32, 1 = BF16, 2 = FP16) and kernel family (0 = binned sweeps, 1 =
# tiles, blocks, batches, refresh), so the instantiations compile in parallel.
CU_VARIANTS = [("launch.cu", rt, part) for rt in (0, 1, 2) for part in (0, 1)]
CXX_SOURCES = ["synth.cpp", "relabel.cpp", "blocked.cpp"]
CLI_SOURCES = ["cli/main.cpp", "cli/loader.cpp"]


def _run_parallel(cmds):
    procs = [(c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)) for c in cmds]
    failed = []
    for c, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((c, out.decode(errors="replace")))
    if failed:
        msg = "\n".join(" ".join(c) + "\n" + o for c, o in failed)
        raise RuntimeError("native build failed:\n" + msg)


def build(verbose=False, with_cli=True):
    """Compiles every translation unit and links the library and the CLI."""
    obj_dir = OBJDIR
    lib = LIB
    os.makedirs(obj_dir, exist_ok=True)
    os.makedirs(os.path.dirname(lib), exist_ok=True)
    os.makedirs(BINDIR, exist_ok=True)
    cmds, objs = [], []
    for src in CU_SOURCES:
        obj = os.path.join(obj_dir, os.path.basename(src) + ".o")
        cmds.append([NVCC] + NVFLAGS + ["-c", os.path.join(CSRC, src), "-o", obj])
        objs.append(obj)
    for src, rt, part in CU_VARIANTS:
        obj = os.path.join(obj_dir, "launch_rt%d_part%d.o" % (rt, part))
        cmds.append([NVCC] + NVFLAGS + ["-DCDMF_LAUNCH_RT=%d" % rt, "-DCDMF_LAUNCH_PART=%d" % part,
                                        "-c", os.path.join(CSRC, src), "-o", obj])
        objs.append(obj)
    for src in CXX_SOURCES:
        obj = os.path.join(obj_dir, os.path.basename(src) + ".o")
        cmds.append(["g++"] + CXXFLAGS + ["-c", os.path.join(CSRC, src), "-o", obj])
        objs.append(obj)
    cli_objs = []
    for src in (CLI_SOURCES if with_cli else []):
        path = os.path.join(CSRC, src)
        if not os.path.exists(path):
            continue
        obj = os.path.join(OBJDIR, "cli_" + os.path.basename(src) + ".o")
        cmds.append(["g++"] + CXXFLAGS + ["-c", path, "-o", obj])
        cli_objs.append(obj)
    if verbose:
        for c in cmds:
            print(" ".join(c), file=sys.stderr)
    _run_parallel(cmds)
    tmp = lib + ".tmp"
    _run_parallel([[NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-Xcompiler", "-fopenmp", "-lgomp",
                                                         "-Xlinker", "--no-undefined"]])
    os.replace(tmp, lib)
    if cli_objs:
        _run_parallel([["g++", "-o", CLI] + cli_objs + ["-L", LIBDIR, "-lcdmf_cuda", "-Wl,-rpath,$ORIGIN/../lib",
                                                         "-fopenmp"]])
    return lib
