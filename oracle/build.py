"""Build the CPU oracle ``oracle/_ref/libmqref.so`` (test infrastructure only).

gcc, ``-ffp-contract=off`` so every host (x86-64, aarch64) evaluates the same rounded
operations and the oracle's results are reproducible bit for bit.
"""
from __future__ import annotations

import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref" / "libmqref.so"


def build() -> Path:
    OUT.parent.mkdir(exist_ok=True)
    srcs = [HERE / "mqref.c", HERE / "mqtandem.c"]
    deps = srcs + [HERE / "mqref.h", HERE / "mqtandem.h"]
    if OUT.exists() and OUT.stat().st_mtime > max(p.stat().st_mtime for p in deps):
        return OUT
    tmp = OUT.with_suffix(".tmp.so")
    subprocess.run(["gcc", "-O2", "-std=c11", "-Wall", "-ffp-contract=off", "-fPIC", "-pthread", "-shared",
                    *map(str, srcs), "-o", str(tmp), "-lm"], check=True, capture_output=True)
    tmp.replace(OUT)
    return OUT


if __name__ == "__main__":
    print(build())
