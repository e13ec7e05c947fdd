"""Build recipe of the oracle (test infrastructure only): compiles
``oracle/pg_oracle.cpp`` (the fluid path), ``oracle/unet_oracle.cpp`` (the
learned pressure guess) and ``oracle/wavelet_oracle.cpp`` (the wavelet
transforms) with g++ into ``oracle/_build/libpg_oracle.so``.

-ffp-contract=off keeps a*b+c unfused on every host (aarch64 gcc fuses by
default), so float results match a sequential evaluation of the reference.
The reference itself (Rust, crates.io dependencies not vendored) cannot be
built in this environment, so there is no ``oracle/_ref``.
"""

import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRCS = [os.path.join(HERE, f) for f in ("pg_oracle.cpp", "unet_oracle.cpp", "wavelet_oracle.cpp")]
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libpg_oracle.so")
FLAGS = ["-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-std=c++17", "-shared"]


def build(force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    digest = hashlib.sha256(b"".join(open(f, "rb").read() for f in SRCS) + " ".join(FLAGS).encode()).hexdigest()
    stamp = LIB + ".stamp"
    if not force and os.path.exists(LIB) and os.path.exists(stamp) and open(stamp).read() == digest:
        return LIB
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    tmp = LIB + ".tmp"
    subprocess.run([cxx] + FLAGS + ["-o", tmp] + SRCS, check=True)
    os.replace(tmp, LIB)
    with open(stamp, "w") as f:
        f.write(digest)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
