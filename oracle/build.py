"""Build recipes for the oracle and the compiled reference (TEST INFRASTRUCTURE)."""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_ORACLE = os.path.join(HERE, "_build", "libswm_oracle.so")
REF_DIR = os.path.join(HERE, "_ref")
LIB_SWREF = os.path.join(REF_DIR, "libswref.so")


def reference_tree() -> str:
    """The reference's source tree: $REF_DIR, else a directory named
    `reference` beside this repository's root (the same rule as build_ref.sh)."""
    return os.environ.get("REF_DIR") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")


def _newer(target, deps):
    return os.path.exists(target) and all(os.path.getmtime(d) <= os.path.getmtime(target) for d in deps)


def build_oracle() -> str:
    src = os.path.join(HERE, "swm_oracle.c")
    os.makedirs(os.path.dirname(LIB_ORACLE), exist_ok=True)
    if not _newer(LIB_ORACLE, [src, os.path.join(HERE, "swm_oracle.h")]):
        p = subprocess.run(["gcc", "-O2", "-fPIC", "-shared", "-std=gnu11", "-pthread", src, "-o", LIB_ORACLE],
                           capture_output=True, text=True)
        if p.returncode:
            sys.stderr.write(p.stdout + p.stderr)
            raise RuntimeError("oracle build failed")
    return LIB_ORACLE


def build_ref() -> str | None:
    """Compile the reference's own source into oracle/_ref (see build_ref.sh).

    Works where the reference tree is present, or where oracle/_ref/src was
    produced earlier; returns None when neither is available.
    """
    have_src = os.path.exists(os.path.join(REF_DIR, "src", "mapper_ref.c"))
    have_tree = os.path.exists(os.path.join(reference_tree(), "mapper_cpe.c"))
    if not (have_src or have_tree):
        return None
    if have_src and os.path.exists(LIB_SWREF) and not have_tree:
        return LIB_SWREF
    p = subprocess.run(["bash", os.path.join(HERE, "build_ref.sh")], capture_output=True, text=True)
    if p.returncode != 0:
        sys.stderr.write(p.stdout + p.stderr)
        return None
    return LIB_SWREF


def build_all() -> None:
    build_oracle()
    build_ref()
