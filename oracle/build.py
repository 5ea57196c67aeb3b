"""Build recipe of the CPU oracle (test infrastructure only).

build_oracle() compiles oracle/slo.cpp, the CPU restatement of SoftLight's
draw path, into oracle/build/libslo.so with FP contraction off, so it gives
identical results on x86-64 and aarch64. Only the tests, the smoke check and
the benchmark's CPU-baseline leg load it.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "build")
LIB = os.path.join(BUILD, "libslo.so")

CXXFLAGS = ["-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
            "-Wall", "-Wextra", "-pthread"]


def build_oracle(force=False):
    src = os.path.join(HERE, "slo.cpp")
    deps = [src, os.path.join(HERE, "slo.h"), os.path.join(HERE, "..", "include", "slg.h"),
            os.path.join(HERE, "..", "include", "slg_programs.h"),
            os.path.join(HERE, "..", "include", "slg_half.h"), __file__]
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(d) for d in deps):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".tmp"
    res = subprocess.run(["g++", *CXXFLAGS, "-o", tmp, src], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build_oracle(force=True))
