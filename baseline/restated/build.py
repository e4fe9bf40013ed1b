"""Builds the restated reference traversal and path tracer (baseline/restated/*.cu) into
baseline/restated/_build/librefkernel.so: default nvcc optimisation flags
(FMA contraction on, as the reference's build has), relocatable device code
with the AABB, triangle and BVH functions in separate translation units
(the reference's CUDA_SEPARABLE_COMPILATION), sm_103a.  A measurement
comparator for bench.py; not part of the product."""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "librefkernel.so")
SRC = ["ref_aabb.cu", "ref_triangle.cu", "ref_bvh.cu", "ref_path.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
ROOT = os.path.dirname(os.path.dirname(HERE))
CSRC = os.path.join(ROOT, "craystal_gb300", "csrc")
INCLUDES = ["-I", os.path.join(ROOT, "include"), "-I", CSRC]


def build(force=False):
    deps = [os.path.join(HERE, f) for f in SRC + ["ref_common.cuh", "build.py"]]
    deps += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in deps):
        return LIB
    os.makedirs(OUT, exist_ok=True)
    objs = []
    for f in SRC:
        o = os.path.join(OUT, f.replace(".cu", ".o"))
        subprocess.run(["nvcc", *ARCH, "-std=c++17", "-rdc=true", "-Xcompiler", "-fPIC", *INCLUDES, "-c",
                        os.path.join(HERE, f), "-o", o], check=True)
        objs.append(o)
    dlink = os.path.join(OUT, "dlink.o")
    subprocess.run(["nvcc", *ARCH, "-dlink", "-Xcompiler", "-fPIC", *objs, "-o", dlink], check=True)
    subprocess.run(["nvcc", *ARCH, "-shared", *objs, dlink, "-o", LIB], check=True)
    return LIB


if __name__ == "__main__":
    print(build("--force" in sys.argv))
