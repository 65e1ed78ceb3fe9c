"""Builds the oracle's C restatement (oracle/_build/libamdat_oracle.so) and the
reference AMDAT binary (oracle/_ref/<machine>/AMDAT via oracle/ref.mk) from the
reference's own sources.  Test infrastructure only: the checker of the parity
tests and the timed CPU reference of the benchmark.

Where the reference sources are: the directory named by AMDAT_REFERENCE, else
the git-ignored source copy baseline/_ref/src that
    python oracle/build_oracle.py --stage-sources <AMDAT checkout>
makes (src/, the two vendored libraries and VERSION, copied unmodified).  The
copy is never committed; it travels with the working tree to machines that
have no reference checkout, where the benchmark's reference arm compiles it.
"""
from __future__ import annotations

import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
LIB = os.path.join(HERE, "_build", "libamdat_oracle.so")
STAGED = os.path.join(REPO, "baseline", "_ref", "src")
# the parts of the reference tree the binary is built from
STAGE_PARTS = ("src", os.path.join("third_party", "voro++-0.4.6"),
               os.path.join("third_party", "xdrfile-1.1b"), "VERSION")


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


def reference_source() -> str | None:
    """The reference source tree: AMDAT_REFERENCE, else the staged copy."""
    for d in (os.environ.get("AMDAT_REFERENCE"), STAGED):
        if d and os.path.isdir(os.path.join(d, "src")):
            return d
    return None


def stage_sources(ref: str) -> str:
    """Copy the reference parts the build needs into baseline/_ref/src (git-ignored)."""
    if not os.path.isdir(os.path.join(ref, "src")):
        raise SystemExit(f"{ref} is not an AMDAT source tree")
    tmp = STAGED + f".tmp{os.getpid()}"
    for part in STAGE_PARTS:
        src, dst = os.path.join(ref, part), os.path.join(tmp, part)
        os.makedirs(os.path.dirname(dst), exist_ok=True)
        if os.path.isdir(src):
            shutil.copytree(src, dst)
        else:
            shutil.copyfile(src, dst)
    for root, dirs, files in os.walk(tmp):
        for n in dirs + files:
            p = os.path.join(root, n)
            os.chmod(p, os.stat(p).st_mode | 0o200)
    if os.path.isdir(STAGED):
        shutil.rmtree(STAGED)
    os.replace(tmp, STAGED)
    return STAGED


def reference_binary_path() -> str:
    return os.path.join(HERE, "_ref", platform.machine(), "AMDAT")


def build_reference(jobs: int | None = None) -> str | None:
    """Compile the reference from its own sources when they are present (the
    binary of this machine's architecture, under oracle/_ref/<machine>/)."""
    ref = reference_source()
    if ref is None:
        return None
    out = os.path.dirname(reference_binary_path())
    binary = reference_binary_path()
    if os.path.exists(binary):
        return binary
    jobs = jobs or min(32, os.cpu_count() or 4)
    subprocess.run(["make", "-f", os.path.join(HERE, "ref.mk"), f"REF={os.path.abspath(ref)}",
                    f"OUT={out}", f"-j{jobs}"], check=True, cwd=REPO,
                   stdout=subprocess.DEVNULL)
    return binary


if __name__ == "__main__":
    if "--stage-sources" in sys.argv:
        print(stage_sources(sys.argv[sys.argv.index("--stage-sources") + 1]))
    print(build_lib(force="--force" in sys.argv))
    print(build_reference())
