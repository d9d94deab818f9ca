"""Microbenchmark of the front-update GEMM C -= A B (complex64, row-major)
through the tcgen05 kernel (path 1), the SIMT kernel (path 0) or the
tall-skinny SIMT kernel of the solves (path 2, N <= 32) or the tall-skinny
tcgen05 kernel of the solves (path 3, N <= 32; A by TMA when aligned, path 6
with A always copied by the loader warps), on random operands
resident on the device:

    python -m wtomo3d_gb300.gemm_bench M N K [--path 1] [--reps 5]

Prints one JSON line with the mean launch time, the real-flop rate 8 M N K / t
and the rate at which A (8 M K bytes) is read.  The tensor-core timing excludes the operand split, which the
factorisation runs as a separate kernel.
"""
import argparse
import ctypes
import json
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("M", type=int)
    ap.add_argument("N", type=int)
    ap.add_argument("K", type=int)
    ap.add_argument("--path", type=int, default=1, choices=[0, 1, 2, 3, 6])
    ap.add_argument("--reps", type=int, default=5)
    a = ap.parse_args()
    import wtomo3d_gb300 as wt
    L = wt.lib()
    L.wt3d_bench_gemm.argtypes = [ctypes.c_int] * 5 + [ctypes.c_void_p]
    ms = ctypes.c_double()
    rc = L.wt3d_bench_gemm(a.path, a.M, a.N, a.K, a.reps, ctypes.byref(ms))
    if rc:
        raise SystemExit("wt3d_bench_gemm failed (%d): %s" % (rc, L.wt3d_last_error().decode()))
    fl = 8.0 * a.M * a.N * a.K
    print(json.dumps({"M": a.M, "N": a.N, "K": a.K, "path": {0: "simt", 1: "tcgen05", 2: "simt-tall-skinny", 3: "tcgen05-tall-skinny", 6: "tcgen05-tall-skinny-copies"}[a.path], "ms": ms.value,
                      "tflops": fl / ms.value / 1e9, "a_gbs": 8.0 * a.M * a.K / ms.value / 1e6}))


if __name__ == "__main__":
    main()
