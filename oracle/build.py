"""Build recipe of the oracle (test infrastructure only).

Compiles oracle/irlba_oracle.cpp, the plain-C++ restatement of CppIrlba's
IRLBA path, into oracle/_build/liboracle.so with g++ and OpenMP, together with
the seeded synthetic-input generator (cppirlba_gb300/csrc/datagen.cpp), so that
the timed CPU reference run generates its input without loading any library of
the product. The reference itself is not built: it needs Eigen 5.0.0, aarand,
subpar and sanisizer, none of which is available offline.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "irlba_oracle.cpp")
GEN = os.path.join(os.path.dirname(HERE), "cppirlba_gb300", "csrc", "datagen.cpp")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")


def build(force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC), os.path.getmtime(GEN)):
        return LIB
    cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-pthread", "-ffp-contract=off", SRC, GEN,
           "-o", LIB]
    res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + res.stdout)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
