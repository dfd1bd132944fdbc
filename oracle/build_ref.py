"""Compile the reference's own face-pair cubature (C++) for the oracle tests.

The source is compiled where it lies (the reference checkout, path given by
VOXSCATTER_REFERENCE or the default below) together with oracle/ref_nop_glue.cpp;
the library goes to oracle/_ref/libref_nop.so (git-ignored).  Nothing from the
reference is copied into this repository.  Returns the library path, or None
when the reference checkout or g++ is absent."""
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("VOXSCATTER_REFERENCE", "/root/reference")
SRC = os.path.join(REF, "src", "src_vie", "src_operators", "mexcubatures", "cubature_nop_const.cpp")
OUT = os.path.join(HERE, "_ref", "libref_nop.so")


def build(verbose=False):
    if not os.path.exists(SRC) or shutil.which("g++") is None:
        return OUT if os.path.exists(OUT) else None
    glue = os.path.join(HERE, "ref_nop_glue.cpp")
    if os.path.exists(OUT) and os.path.getmtime(OUT) >= max(os.path.getmtime(SRC), os.path.getmtime(glue)):
        return OUT
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    cmd = ["g++", "-O2", "-shared", "-fPIC", "-o", OUT, glue, SRC]
    subprocess.run(cmd, check=True, capture_output=not verbose)
    return OUT


if __name__ == "__main__":
    print(build(verbose=True))
