"""Build the C oracle (oracle_cpu.c) into oracle/_build/liboracle_cpu.so with gcc
(test infrastructure and CPU baseline only).  No architecture-specific flags,
so the same source builds on x86_64 and aarch64."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build", "liboracle_cpu.so")


def build():
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    cmd = ["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-o", OUT + ".tmp",
           os.path.join(HERE, "oracle_cpu.c"), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    print(build())
