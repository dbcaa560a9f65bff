"""Build recipe of the checkers under oracle/ (test infrastructure; nothing in the product links them).

    python oracle/build.py [reference source dir]

build_oracle():    liboracle.so from jsb_oracle.cpp (the CPU restatement of the soft-body step), with
                   -ffp-contract=off like the reference's deterministic build.
build_reference(): the reference itself (Jolt Physics) from its own sources into oracle/_ref/ with
                   Makefile.ref, only where those sources are present (never on the GPU hosts).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
ORACLE_SRC = os.path.join(HERE, "jsb_oracle.cpp")
ORACLE_LIB = os.path.join(HERE, "liboracle.so")


def build_oracle() -> str:
    if not os.path.exists(ORACLE_LIB) or os.path.getmtime(ORACLE_LIB) < os.path.getmtime(ORACLE_SRC):
        subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-pthread", ORACLE_SRC, "-o",
                        ORACLE_LIB], check=True)
    return ORACLE_LIB


def build_reference(ref: str | None, jobs: int | None = None) -> bool:
    """Builds oracle/_ref from the reference sources at `ref`; False when they are absent."""
    if not ref or not os.path.isdir(os.path.join(ref, "Jolt")) or shutil.which("make") is None:
        return False
    j = str(jobs or os.cpu_count() or 4)
    subprocess.run(["make", "-f", os.path.join("oracle", "Makefile.ref"), f"REF={ref}", f"-j{j}"], cwd=REPO, check=True,
                   stdout=subprocess.DEVNULL)
    return True


if __name__ == "__main__":
    print(build_oracle())
    if len(sys.argv) > 1:
        print("reference built:", build_reference(sys.argv[1]))
