"""Builds the oracle's C restatement (oracle/_build/libamdat_oracle.so) and,
when the reference AMDAT source tree is present, the reference binary
(oracle/_ref/AMDAT via oracle/ref.mk).  Test infrastructure only."""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
LIB = os.path.join(HERE, "_build", "libamdat_oracle.so")
REF_BIN = os.path.join(HERE, "_ref", "AMDAT")
REF_SRC = os.environ.get("AMDAT_REFERENCE", "/root/reference")


def build_lib(force: bool = False) -> str:
    src = os.path.join(HERE, "amdat_oracle.c")
    hdr = os.path.join(HERE, "amdat_oracle.h")
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    tmp = LIB + f".tmp{os.getpid()}"
    # -ffp-contract=off keeps the reference's uncontracted FP32 roundings on aarch64 too
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           src, "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


def build_reference(jobs: int = 8) -> str | None:
    """Compile the reference from its own sources when they are present."""
    if not os.path.isdir(os.path.join(REF_SRC, "src")):
        return None
    if os.path.exists(REF_BIN):
        return REF_BIN
    subprocess.run(["make", "-f", os.path.join(HERE, "ref.mk"), f"REF={REF_SRC}",
                    f"OUT={os.path.join(HERE, '_ref')}", f"-j{jobs}"], check=True, cwd=REPO,
                   stdout=subprocess.DEVNULL)
    return REF_BIN


if __name__ == "__main__":
    print(build_lib(force="--force" in sys.argv))
    print(build_reference())
