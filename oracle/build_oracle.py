"""Build recipe for the oracle (test infrastructure): the FP64 CPU restatement
in visacd_oracle.cpp -> oracle/liboracle.so (g++, OpenMP, -ffp-contract=off so
the written operation order is the executed one)."""
from __future__ import annotations

import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
SRC = HERE / "visacd_oracle.cpp"


def build(force: bool = False) -> Path:
    if force or not LIB.exists() or SRC.stat().st_mtime > LIB.stat().st_mtime:
        cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
               "-o", str(LIB), str(SRC)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(force=True))
