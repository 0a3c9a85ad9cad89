"""Build the oracle's C restatement (test infrastructure only).

``oracle/flux_total.c`` (the per-particle FP64 flux total) is compiled with
the host C compiler into ``oracle/libmartini_oracle.so``.  Only the tests,
``__graft_entry__.smoke()`` and the bench's CPU legs load it, as the checker.
"""

from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "flux_total.c")
LIB = os.path.join(HERE, "libmartini_oracle.so")


def build(force: bool = False) -> str:
    """Compile the C oracle if it is missing or older than its source."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cc = os.environ.get("CC") or shutil.which("gcc") or shutil.which("cc")
    if not cc:
        raise RuntimeError("no C compiler for the oracle's C restatement")
    tmp = LIB + f".{os.getpid()}.tmp"
    cmd = [cc, "-O2", "-std=c99", "-fPIC", "-shared", "-o", tmp, SRC, "-lm", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle C build failed:\n{' '.join(cmd)}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
