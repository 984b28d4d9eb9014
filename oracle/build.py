"""Build recipe for the CPU oracle (test infrastructure, never shipped).

Two builds of oracle/sflow_oracle.c:
  libsflow_oracle.so       the parity build: FP64 with no FMA contraction
                           (-ffp-contract=off, -fno-fast-math) so that the
                           operation order of the restatement is what runs
  libsflow_oracle_fast.so  the timing build for the CPU baseline: the
                           reference's own compiler flags (src/Makefile.am:22,
                           -fopenmp -Ofast -funroll-all-loops); its results
                           are not used as a checker
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "sflow_oracle.c")
LIB = os.path.join(HERE, "libsflow_oracle.so")
LIB_FAST = os.path.join(HERE, "libsflow_oracle_fast.so")
DEPS = [SRC, os.path.join(HERE, "..", "include", "sflow.h"),
        os.path.join(HERE, "..", "imex_sflow2d_dev_gb300", "csrc", "sflow_math.h")]
PARITY_FLAGS = ["-O2", "-ffp-contract=off", "-fno-fast-math"]
TIMING_FLAGS = ["-Ofast", "-funroll-all-loops"]   # + -fopenmp, as the reference


def _build(out, flags, force, verbose):
    if (not force and os.path.exists(out)
            and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in DEPS)):
        return out
    cmd = ["gcc"] + flags + ["-std=gnu11", "-fPIC", "-shared", "-fopenmp", "-Wall",
                             "-Wno-unused-function", "-o", out + ".tmp", SRC, "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(out + ".tmp", out)
    return out


def build_oracle(force=False, verbose=False):
    """Both builds; returns the parity build's path."""
    _build(LIB_FAST, TIMING_FLAGS, force, verbose)
    return _build(LIB, PARITY_FLAGS, force, verbose)


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv, verbose=True))
