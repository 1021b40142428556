"""Build recipe for the oracle (test infrastructure only).

* ``liboracle.so``   — the CPU FP64 restatement (staqdic_oracle.cpp), OpenMP.
* ``_ref/libba_interp2_ref.so`` — the reference's own ``ba_interp2.cpp``,
  compiled unmodified from the reference checkout against ``mexshim/mex.h``.
  It is built only when the reference checkout is present; outputs go to
  ``oracle/_ref/`` (git-ignored).

``-ffp-contract=off`` keeps every multiply and add separately rounded, the way
the reference's C++ is evaluated on x86-64 without FMA, so the oracle gives the
same bits on x86-64 and on aarch64.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# The STAQ-DIC checkout whose ba_interp2.cpp is compiled: STAQDIC_REFERENCE,
# else the read-only mount where this recipe's build environment keeps it.
# Where neither exists the reference checker is simply not built.
REF_SRC = os.environ.get("STAQDIC_REFERENCE") or "/root/reference"

CXXFLAGS = ["-O3", "-fPIC", "-shared", "-ffp-contract=off", "-std=c++17"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("oracle build failed: " + " ".join(cmd))


def oracle_lib_path():
    return os.path.join(HERE, "liboracle.so")


def ref_lib_path():
    return os.path.join(HERE, "_ref", "libba_interp2_ref.so")


def build_oracle(force=False):
    out = oracle_lib_path()
    src = os.path.join(HERE, "staqdic_oracle.cpp")
    if not force and os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
        return out
    _run(["g++", *CXXFLAGS, "-fopenmp", "-o", out, src])
    return out


def build_ref(force=False):
    """Compile the reference's ba_interp2.cpp if the reference tree exists."""
    src = os.path.join(REF_SRC, "ba_interp2.cpp")
    if not os.path.exists(src):
        return None
    out = ref_lib_path()
    shim = os.path.join(HERE, "mexshim", "mexshim.cpp")
    if not force and os.path.exists(out) and os.path.getmtime(out) >= max(
            os.path.getmtime(src), os.path.getmtime(shim)):
        return out
    os.makedirs(os.path.dirname(out), exist_ok=True)
    _run(["g++", *CXXFLAGS, "-I", os.path.join(HERE, "mexshim"), "-o", out, src, shim])
    return out


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_ref(force=True))
