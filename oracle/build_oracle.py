"""Build recipe for the CPU oracle (test infrastructure only).

Compiles ``oracle/jmul_oracle.c`` into ``oracle/_build/liboracle.so`` with gcc.
``-ffp-contract=off`` keeps every multiply and add separately rounded except the
explicit ``fma()`` calls, which is what makes the oracle's per-element operation
order equal to jBLAS's ``d = a1*x1; d = fma(ak, xk, d)`` chain.  On x86_64 hosts
with the FMA extension ``-mfma`` lets the compiler use the hardware instruction
for ``fma()`` (the result is identical, it is only faster); on aarch64 the
instruction is part of the base ISA.
"""
import os
import platform
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "jmul_oracle.c")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")


def _cpu_has(flag):
    try:
        with open("/proc/cpuinfo") as f:
            return any(flag in line.split() for line in f if line.startswith("flags"))
    except OSError:
        return False


def build(force=False, verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(SRC)
            and os.path.getmtime(LIB) >= os.path.getmtime(__file__)):
        return LIB
    cmd = ["gcc", "-O3", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-fno-math-errno", "-std=c11"]
    if platform.machine() in ("x86_64", "AMD64") and _cpu_has("fma") and _cpu_has("avx2"):
        cmd += ["-mfma", "-mavx2"]
        if _cpu_has("avx512f"):
            cmd += ["-mavx512f"]   # the 32-register file pick_kernel_size sizes the tile for
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd += [SRC, "-o", tmp, "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
