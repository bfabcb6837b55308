"""Build recipe for the oracle (test infrastructure only).

``build_oracle()`` compiles oracle/oracle.c (the C restatement) into
oracle/_build/liboracle.so with gcc; ``build_ref()`` compiles the unmodified
reference headers into oracle/_ref/libpwmref.so when the reference tree is
present (development container only; see build_ref.sh).
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libpwmref.so")
REF_STATS = os.path.join(HERE, "_ref", "calc_stats")
REF_DIR = os.environ.get("PWM_REFERENCE_DIR", "/root/reference")


def build_oracle(force=False):
    src = [os.path.join(HERE, "oracle.c")]
    hdr = os.path.join(HERE, "oracle.h")
    if not force and os.path.exists(LIB):
        newest = max(os.path.getmtime(p) for p in src + [hdr])
        if os.path.getmtime(LIB) >= newest:
            return LIB
    os.makedirs(BUILD, exist_ok=True)
    cmd = ["gcc", "-O2", "-std=c11", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           "-o", LIB] + src + ["-lm"]
    subprocess.check_call(cmd)
    return LIB


def build_ref(force=False):
    """Compile oracle/_ref from the reference tree; returns the path or None."""
    if not os.path.isdir(os.path.join(REF_DIR, "Matrix")):
        return None
    if not force and os.path.exists(REF_LIB):
        srcs = [os.path.join(HERE, "ref_harness.cpp"), os.path.join(HERE, "ref_stats_main.cpp"),
                os.path.join(HERE, "build_ref.sh")]
        outs = [REF_LIB, REF_STATS]
        if all(os.path.exists(o) for o in outs) and \
                min(os.path.getmtime(o) for o in outs) >= max(os.path.getmtime(p) for p in srcs):
            return REF_LIB
    subprocess.check_call(["sh", os.path.join(HERE, "build_ref.sh")])
    return REF_LIB


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_ref(force=True))
