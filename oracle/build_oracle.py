"""Build the oracle's C helper (``packed_decode.c`` -> ``liboracle.so``).

Test infrastructure only: the helper speeds up the FP64 oracle's decode of
large packed matrices; the product library never links it."""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
SOURCES = [HERE / "packed_decode.c"]


def build(force: bool = False) -> Path:
    if not force and LIB.exists() and all(s.stat().st_mtime <= LIB.stat().st_mtime for s in SOURCES):
        return LIB
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        raise RuntimeError("no C compiler for the oracle helper")
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cc, "-O2", "-std=c99", "-shared", "-fPIC", "-pthread", *map(str, SOURCES), "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle helper build failed:\n{r.stdout}\n{r.stderr}")
    tmp.replace(LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
