"""Build recipe for the oracle (test infrastructure only).

Compiles oracle/perm_oracle.cpp (double-double restatement) and
oracle/perm_port.cpp (the reference's CPU method in its own arithmetic, used as
the timed CPU baseline) into oracle/_build/libpqoracle.so, and — where the
reference source tree is present — the reference's own module into oracle/_ref/
through oracle/build_ref.sh.  Host code only; builds the same on x86 and Arm.
"""

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD_DIR, "libpqoracle.so")


def build(force: bool = False, with_reference: bool = True) -> str:
    os.makedirs(BUILD_DIR, exist_ok=True)
    srcs = [os.path.join(HERE, "perm_oracle.cpp"), os.path.join(HERE, "perm_port.cpp")]
    stale = force or not os.path.exists(LIB) or any(
        os.path.getmtime(s) > os.path.getmtime(LIB) for s in srcs
    )
    if stale:
        objs = []
        # the double-double restatement: no contraction, so TwoSum/TwoProduct stay exact
        flags = {
            srcs[0]: ["-O2", "-ffp-contract=off"],
            # the port mirrors the reference's Release build flags
            srcs[1]: ["-O3"],
        }
        procs = []
        for s in srcs:
            o = os.path.join(BUILD_DIR, os.path.basename(s) + ".o")
            objs.append(o)
            cmd = ["g++", "-std=c++17", "-fopenmp", "-fPIC", "-c", s, "-o", o] + flags[s]
            procs.append(subprocess.Popen(cmd))
        for p in procs:
            if p.wait() != 0:
                raise RuntimeError("oracle build failed")
        tmp = LIB + ".tmp"
        subprocess.check_call(["g++", "-shared", "-fopenmp", "-o", tmp] + objs)
        os.replace(tmp, LIB)
    if with_reference:
        script = os.path.join(HERE, "build_ref.sh")
        ref_lib_dir = os.path.join(HERE, "_ref", "piquasso", "_math")
        have_ref = os.path.isdir(ref_lib_dir) and any(
            f.startswith("permanent") and f.endswith(".so") for f in os.listdir(ref_lib_dir)
        )
        if not have_ref:
            subprocess.call(["bash", script], env=dict(os.environ, PYTHON=sys.executable))
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
