"""Builds the oracle restatement oracle/port/ldlt_port.cpp into
oracle/_port/libnqport.so (plain g++, no GPU).  Test infrastructure: only the
tests, the smoke check and the benchmark's CPU baseline load it."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "port", "ldlt_port.cpp")
OUT = os.path.join(HERE, "_port", "libnqport.so")


def build() -> str:
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    if os.path.exists(OUT) and os.path.getmtime(OUT) >= os.path.getmtime(SRC):
        return OUT
    cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", SRC, "-o", OUT, "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    return OUT


if __name__ == "__main__":
    print(build())
