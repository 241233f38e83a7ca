"""Build of the GB300 SunlightLB shared library, in tree.

``build()`` compiles the CUDA device layer (csrc/cuda, sm_103a) and the host
C implementation of the SunlightLB API (csrc/host) into
``sunlightlb_gb300/lib/libsunlightlb.so`` (soname libsunlightlb.so.1, the
reference's soname).  Translation units compile in parallel; nothing is
installed outside the package directory.
"""

import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
INC = os.path.join(ROOT, "include")
CUDA_DIR = os.path.join(PKG, "csrc", "cuda")
HOST_DIR = os.path.join(PKG, "csrc", "host")
LIB_DIR = os.path.join(PKG, "lib")
OBJ_DIR = os.path.join(LIB_DIR, "obj")
LIB = os.path.join(LIB_DIR, "libsunlightlb.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + INC, "-I" + CUDA_DIR]
# FP64 kernels: no FMA contraction, so FP64 results equal the reference's
PER_FILE = {"slbc_f64.cu": ["-fmad=false"], "slbc_noalloc.cu": ["-fmad=false"]}
# host C: strict IEEE double (no contraction, which gcc applies on aarch64)
CC_FLAGS = ["-O2", "-fPIC", "-std=gnu99", "-Wall", "-Wno-unused-result", "-Werror=implicit-function-declaration",
            "-fno-fast-math", "-ffp-contract=off", "-I" + INC, "-I" + HOST_DIR]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the GB300 SunlightLB library needs the CUDA toolkit")


def _sources():
    cu = sorted(f for f in os.listdir(CUDA_DIR) if f.endswith(".cu"))
    c = sorted(f for f in os.listdir(HOST_DIR) if f.endswith(".c"))
    return cu, c


def _deps(directory, ext):
    return [os.path.join(directory, f) for f in os.listdir(directory) if f.endswith(ext)]


def _newest(paths):
    return max((os.path.getmtime(p) for p in paths if os.path.exists(p)), default=0.0)


def up_to_date():
    if not os.path.exists(LIB):
        return False
    cu, c = _sources()
    srcs = ([os.path.join(CUDA_DIR, f) for f in cu] + [os.path.join(HOST_DIR, f) for f in c]
            + _deps(CUDA_DIR, ".cuh") + _deps(HOST_DIR, ".h") + _deps(INC, ".h")
            + [os.path.abspath(__file__)])
    return os.path.getmtime(LIB) >= _newest(srcs)


def build(force=False, verbose=False):
    """Compile every translation unit (in parallel) and link the library."""
    if not force and up_to_date():
        return LIB
    os.makedirs(OBJ_DIR, exist_ok=True)
    nvcc = _nvcc()
    cu, c = _sources()
    jobs = []
    objs = []
    for f in cu:
        obj = os.path.join(OBJ_DIR, f[:-3] + ".o")
        cmd = [nvcc] + ARCH + NVCC_FLAGS + PER_FILE.get(f, []) + ["-c", os.path.join(CUDA_DIR, f), "-o", obj]
        jobs.append(cmd)
        objs.append(obj)
    cc = os.environ.get("CC", "gcc")
    for f in c:
        obj = os.path.join(OBJ_DIR, f[:-2] + ".o")
        jobs.append([cc] + CC_FLAGS + ["-c", os.path.join(HOST_DIR, f), "-o", obj])
        objs.append(obj)
    procs = []
    for cmd in jobs:
        if verbose:
            print(" ".join(cmd))
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for cmd, p in procs:
        out, _ = p.communicate()
        text = out.decode(errors="replace")
        if p.returncode != 0:
            failed.append((cmd, text))
        elif verbose and text.strip():
            print(text)
    if failed:
        msg = "\n".join(" ".join(cmd) + "\n" + text for cmd, text in failed)
        raise RuntimeError("build of libsunlightlb.so failed:\n" + msg)
    tmp = LIB + ".tmp"
    link = [nvcc] + ARCH + ["-shared", "-Xlinker", "-soname=libsunlightlb.so.1",
                            "-Xlinker", "-Bsymbolic", "-Xlinker", "--no-undefined", "-o", tmp] + objs + ["-lm"]
    if verbose:
        print(" ".join(link))
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("link of libsunlightlb.so failed:\n" + r.stdout.decode(errors="replace"))
    os.replace(tmp, LIB)
    return LIB


def build_oracle(with_reference=True, verbose=False):
    """Build the CPU oracle (oracle/liboracle.so) and, where the reference
    sources are present, oracle/_ref (test infrastructure only)."""
    odir = os.path.join(ROOT, "oracle")
    targets = ["all"]
    # the reference's checkout ($SLB_REFERENCE, default /root/reference);
    # oracle/_ref is built only where its sources exist
    ref_src = os.path.join(os.environ.get("SLB_REFERENCE", "/root/reference"), "src")
    if with_reference and os.path.isdir(ref_src):
        targets.append("ref")
    r = subprocess.run(["make", "-s", "-C", odir, "REF_SRC=" + ref_src] + targets,
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if verbose or r.returncode != 0:
        sys.stdout.write(r.stdout.decode(errors="replace"))
    if r.returncode != 0:
        raise RuntimeError("oracle build failed")


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    build_oracle(verbose=True)
    print(LIB)
