"""Recipe for the CPU oracle (test infrastructure): oracle/_build/liboracle.so.

g++ -O2 -std=c++17 -fopenmp -ffp-contract=off -fPIC -shared -I include
    oracle/dem_oracle.cpp -o oracle/_build/liboracle.so

-ffp-contract=off keeps every multiply and add separately rounded, as Julia
evaluates the reference's expressions.  The same recipe is in oracle/Makefile.
"""
from __future__ import annotations

import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
SRC = HERE / "dem_oracle.cpp"
OUT = HERE / "_build" / "liboracle.so"


def build(force: bool = False) -> Path:
    OUT.parent.mkdir(exist_ok=True)
    deps = [SRC, ROOT / "include" / "dem_gb300.h"]
    if force or not OUT.exists() or any(d.stat().st_mtime > OUT.stat().st_mtime for d in deps):
        cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
               "-fPIC", "-shared", f"-I{ROOT / 'include'}", str(SRC), "-o", str(OUT) + ".tmp"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{' '.join(cmd)}\n{res.stderr}")
        Path(str(OUT) + ".tmp").replace(OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
