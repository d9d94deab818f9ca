"""Build recipe for libwtomo3d_gpu.so (sm_103a) and the CPU oracle.

Every translation unit is compiled in parallel with one -gencode (sm_103a)
and linked in-tree into wtomo3d_gb300/libwtomo3d_gpu.so; objects go to
wtomo3d_gb300/_build/.  No cmake, no pip install.  The CUDA toolkit's METIS
(libmetis_static.a) is linked in when a probe program shows that it works.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libwtomo3d_gpu.so")
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "_build", "libwt3d_oracle.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I" + CSRC, "-I" + os.path.join(ROOT, "include")] + ARCH


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def metis_library(nvcc):
    """libmetis_static.a of the CUDA toolkit, if the probe (csrc/metis_probe.c,
    run as its own process) finds METIS_ComputeVertexSeparator working with
    64-bit indices; else None (the general ordering then runs without the
    METIS separator candidate)."""
    import glob
    root = os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    hits = sorted(glob.glob(os.path.join(root, "targets", "*", "lib", "libmetis_static.a")))
    if not hits or shutil.which("gcc") is None:
        return None
    os.makedirs(BUILD, exist_ok=True)
    exe = os.path.join(BUILD, "metis_probe")
    try:
        subprocess.run(["gcc", "-O1", "-o", exe, os.path.join(CSRC, "metis_probe.c"), hits[0], "-lm"],
                       check=True, capture_output=True, timeout=120)
        r = subprocess.run([exe], capture_output=True, text=True, timeout=30)
    except (subprocess.SubprocessError, OSError):
        return None
    return hits[0] if r.returncode == 0 and "metis idx64 ok" in r.stdout else None


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def build_library(verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    metis = metis_library(nvcc)
    flags = NVCC_FLAGS + (["-DWT3D_HAVE_METIS"] if metis else [])
    # objects built with other flags (METIS found or not) are rebuilt
    sig_file = os.path.join(BUILD, "flags.txt")
    sig = " ".join(flags)
    if not os.path.exists(sig_file) or open(sig_file).read() != sig:
        force = True
    srcs = sources()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "wtomo3d_gpu.h"))
    newest_hdr = max(os.path.getmtime(h) for h in headers)
    jobs = []
    objs = []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s) + ".o")
        objs.append(o)
        if force or not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s), newest_hdr):
            jobs.append([nvcc] + flags + ["-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for out in ex.map(_run, jobs):
                if verbose and out.strip():
                    print(out)
    if jobs or not os.path.exists(LIB):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ([metis] if metis else []) + ["-lcudart"])
    with open(sig_file, "w") as f:
        f.write(sig)
    return LIB


def build_oracle():
    os.makedirs(os.path.dirname(ORACLE_LIB), exist_ok=True)
    src = os.path.join(ORACLE_DIR, "wt3d_oracle.c")
    deps = [src, os.path.join(ORACLE_DIR, "asm_impl.inc"), os.path.join(ORACLE_DIR, "wt3d_oracle.h")]
    if not os.path.exists(ORACLE_LIB) or os.path.getmtime(ORACLE_LIB) < max(os.path.getmtime(d) for d in deps):
        _run(["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", src, "-o", ORACLE_LIB, "-lm"])
    return ORACLE_LIB


if __name__ == "__main__":
    print(build_library(verbose=True, force="--force" in sys.argv))
    print(build_oracle())
