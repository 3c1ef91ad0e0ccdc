"""Build recipe for the test oracle (test infrastructure, not the product).

* ``build_oracle()`` compiles the CPU restatement ``og_oracle.c`` into
  ``oracle/_build/libogoracle.so`` (plain C, gcc).
* ``build_ref()`` compiles the reference's own CPU programs from their sources
  where they lie in the reference tree (BFS/cpu_BFS/main.cpp,
  CC/serial/serial.cpp, PR/cpu/pr.cpp), each behind a small harness main from
  ``oracle/ref_harness/``, into ``oracle/_ref/``.  Only possible where the
  reference tree is present; the outputs are git-ignored.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
# the reference tree: $OG_REFERENCE_ROOT, else a directory named "reference"
# beside the repository
DEFAULT_REF_ROOT = os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")

LIB = os.path.join(BUILD, "libogoracle.so")

# harness -> (reference source relative to the reference root, extra flags)
REF_PROGRAMS = {
    "ref_bfs": ("BFS/cpu_BFS/main.cpp", []),
    "ref_cc": ("CC/serial/serial.cpp", []),
    "ref_pr": ("PR/cpu/pr.cpp", []),
}


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


SOURCES = ["og_oracle.c", "og_oracle_rmat.c"]


def build_oracle(force: bool = False) -> str:
    srcs = [os.path.join(HERE, f) for f in SOURCES]
    newest = max(os.path.getmtime(f) for f in srcs + [os.path.join(HERE, "og_oracle.h")])
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    _run(["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fPIC", "-shared", "-Wall", "-o", tmp]
         + srcs + ["-lm", "-lpthread"])
    os.replace(tmp, LIB)
    return LIB


def ref_root() -> str | None:
    root = os.environ.get("OG_REFERENCE_ROOT", DEFAULT_REF_ROOT)
    return root if os.path.isdir(os.path.join(root, "BFS", "cpu_BFS")) else None


def build_ref(force: bool = False) -> dict:
    """Compile the reference CPU programs; returns {name: path} of what exists."""
    root = ref_root()
    out = {}
    if root is None:
        for name in REF_PROGRAMS:
            p = os.path.join(REF_OUT, name)
            if os.path.exists(p):
                out[name] = p
        return out
    os.makedirs(REF_OUT, exist_ok=True)
    harness = os.path.join(HERE, "ref_harness")
    for name, (rel, extra) in REF_PROGRAMS.items():
        dst = os.path.join(REF_OUT, name)
        src = os.path.join(harness, name + ".cpp")
        if not force and os.path.exists(dst) and os.path.getmtime(dst) >= os.path.getmtime(src):
            out[name] = dst
            continue
        cmd = ["g++", "-O2", "-std=c++17", "-w", "-I", harness,
               "-DOG_REF_SRC=\"%s\"" % os.path.join(root, rel),
               "-o", dst, src] + extra
        _run(cmd)
        out[name] = dst
    return out


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
