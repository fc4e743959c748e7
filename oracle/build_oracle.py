"""Build the oracle's C checker (oracle/mc.c -> oracle/_build/libmc_oracle.so).

TEST INFRASTRUCTURE ONLY.  gcc, no -march flags, no FP contraction, so x86 and
Arm builds give identical results.
"""
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libmc_oracle.so")


def build(force=False):
    src = os.path.join(HERE, "mc.c")
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(src):
        return LIB
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        raise RuntimeError("no C compiler for the oracle")
    tmp = LIB + ".tmp"
    subprocess.run([cc, "-O2", "-shared", "-fPIC", "-ffp-contract=off", "-o", tmp, src, "-lm"], check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
