"""Build recipe for the FP64 CPU oracle (test infrastructure only).

Compiles ``numerov_oracle.c`` into ``oracle/libnumerov_oracle.so`` with
``-ffp-contract=off`` so that the only fused multiply-adds are the explicit
``fma()`` calls, which is what makes the FP64 CUDA path bit-comparable to it
on both x86_64 and aarch64 hosts.

The reference (epseon_backend) has no solver code to compile next to it, so
there is no ``oracle/_ref`` build: its only CPU library is a hello-world
module (cpp/cpu/source/libcpu.cpp:3-36) and its gpu library needs the Vulkan
SDK, VMA and fmt submodules that are empty in the mounted tree.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "numerov_oracle.c")
LIB = os.path.join(HERE, "libnumerov_oracle.so")


def build(force: bool = False) -> str:
    """Compile the oracle shared library if it is missing or stale."""
    if (
        not force
        and os.path.exists(LIB)
        and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC), os.path.getmtime(SRC[:-2] + ".h"))
    ):
        return LIB
    cmd = [
        os.environ.get("CC", "gcc"),
        "-O2",
        "-std=c11",
        "-D_GNU_SOURCE",
        "-ffp-contract=off",
        "-fno-fast-math",
        "-fPIC",
        "-shared",
        "-Wall",
        "-o",
        LIB + ".tmp",
        SRC,
        "-lm",
        "-lpthread",
    ]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
