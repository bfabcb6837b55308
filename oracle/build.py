"""Build recipe for the oracle (test infrastructure only).

``build_oracle()`` compiles oracle/oracle.c (the C restatement) into
oracle/_build/liboracle.so with gcc; ``build_ref()`` runs build_ref.sh, which
compiles the unmodified reference headers into oracle/_ref/libpwmref.so when
it finds the reference tree (development container only; on other machines it
builds nothing).  ``reference_dir()`` is the tree the last build used.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libpwmref.so")
REF_STATS = os.path.join(HERE, "_ref", "calc_stats")
REF_DIR_FILE = os.path.join(HERE, "_ref", "reference_dir.txt")


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
    if not force and os.path.exists(REF_LIB) and reference_dir() is not None:
        srcs = [os.path.join(HERE, "ref_harness.cpp"), os.path.join(HERE, "ref_stats_main.cpp"),
                os.path.join(HERE, "build_ref.sh")]
        outs = [REF_LIB, REF_STATS]
        if all(os.path.exists(o) for o in outs) and \
                min(os.path.getmtime(o) for o in outs) >= max(os.path.getmtime(p) for p in srcs):
            return REF_LIB
    subprocess.check_call(["sh", os.path.join(HERE, "build_ref.sh")])
    return REF_LIB if os.path.exists(REF_LIB) and reference_dir() is not None else None


def reference_dir():
    """The reference tree oracle/_ref was built from, or None when it was not
    built or that tree is gone."""
    try:
        with open(REF_DIR_FILE) as f:
            d = f.read().strip()
    except OSError:
        return None
    return d if os.path.isdir(os.path.join(d, "Matrix")) else None


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_ref(force=True))
