"""Builds the test-only host emulation library tests/native/_build/libemul.so."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
CSRC = os.path.join(ROOT, "fcl_gb300", "csrc")
OUT = os.path.join(HERE, "_build", "libemul.so")


def build() -> str:
    srcs = [os.path.join(HERE, "emul.cu"), os.path.join(CSRC, "bvh_build.cpp")]
    deps = srcs + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    if os.path.exists(OUT) and all(os.path.getmtime(OUT) > os.path.getmtime(d) for d in deps):
        return OUT
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    cmd = ["nvcc", "-gencode=arch=compute_103a,code=sm_103a", "-O2", "-std=c++17", "-fmad=false",
           "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", CSRC, "-shared",
           "-x", "cu", srcs[0], "-x", "c++", srcs[1], "-o", OUT, "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("emulation build failed:\n" + r.stdout + r.stderr)
    return OUT


if __name__ == "__main__":
    print(build())
