"""Builds oracle/_ref/libreconref.so from the reference's own sources.

Test infrastructure: the library pins the CPU oracle to the reference's code.
The reference cannot be built as a whole here (OpenCV / GLEW / SDL2 / CUDA
samples headers are missing and its kernels use texture references that CUDA
12+ removed), but its kernels compile for the host once the few CUDA built-ins
they use are provided.  This script

  * copies the named __global__/__device__ functions (and one PhotoTracker
    method) out of the reference's sources (brace matching, read-only) into
    oracle/_ref/frag_<file>.inc,
  * compiles oracle/ref_shim.cpp, which includes those fragments and the
    reference's kernels/kernelUtils.h under a small host shim, together with the
    reference's CPU SE(3) exponential tracker/tracker/expm.c, its 4x4 /
    quaternion helpers tracker/tracker/basic_math.cpp and its result-file
    classes tracker/calib/ResultTxt.cpp and TrackingParams.cpp (wrapped by
    oracle/ref_files.cpp),
  * writes everything only below oracle/_ref/ (git-ignored).

Usage: python oracle/build_ref.py REFERENCE_ROOT   (or $RECON_REFERENCE)
"""
from __future__ import annotations

import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")

# (reference file, [function names]): kernels, and one host method
FRAGMENTS = {
    "tracker/kernels/warp.cu": [
        "interpolateResidualKernel2", "precomputeJacobian4Kernel", "weightJacobianKernel",
        "dotProduct6", "matrixMultVec6", "generateA", "linearFuseKernel", "conjugateGradientKernel",
    ],
    "tracker/kernels/histogram64.cu": ["discretizeResidualKernel", "seekThreshold64Kernel", "generateWeights64Kernel"],
    "tracker/kernels/d2z.cu": [
        "xyz2CloudKernel", "genPointsCloud6Kernel", "computeNormalsCudaKernel", "downSampleCloud6Kernel",
        "extractGradientKernel", "addVertexAttributesWithoutNormalsKernel3", "addVertexAttributesWithoutNormalsKernel4",
        "genOrientedPoints6Kernel", "undistortDisparityKernel", "d2ZLowKernel", "d2ZLowHdrKernel",
    ],
    "tracker/kernels/rgb2gray.cu": [
        "icpResidualKernel2", "icpResidualIndexKernel2", "packIndexKernel", "initWeightsKernel",
        "updateWeightsKernel", "clampWeightsKernel", "convertZMapToXYZKernel", "convertZMapToXYZ6Kernel",
        "rgbTex2GrayHdrZKernel", "rgbdTex2DepthKernel", "rgb2GrayHdrKernel", "rgbF2GrayHdrKernel",
        "convertHdrRGBKernel",
    ],
    # the GPU capture path's RGB undistortion
    "tracker/kernels/undistort.cu": ["undistortHdrRGBKernel"],
    "tracker/kernels/downSample2Cuda.cu": ["fastDownSampleHdrKernel"],
    # one-block kernels with shared memory and __syncthreads (run as 512 host threads)
    "tracker/kernels/filterIndex256.cu": ["seekThreshold256Kernel2", "filterIndexKernel4"],
    # the reconstruction stream: TSDF update, ray cast, shading, resampling
    "tracker/kernels/VoxelGrid_cuda.cu": [
        "transformRT3CUDA", "resetKernel", "initRay", "intersectVoxelGridCuda", "voxelize", "trilinearDensity",
        "trilinearWeight", "estimateLinearZero", "traverseVoxelsCuda", "rayCastVoxelsKernel", "filter3",
        "shadingKernel", "resampleVoxelsKernel", "updateVoxelsKernel", "reconstructionKernel",
    ],
    # the Kinect pre-processing (host routines of the capture path)
    "tracker/multicore/multicore.cpp": [
        "void OMPFunctions::d2Z", "void OMPFunctions::d2ZLow", "void OMPFunctions::convert2Gray",
        "void OMPFunctions::undistort", "void OMPFunctions::undistortLookup",
    ],
    # host code: the keyframe trigger's pose test
    "tracker/tracker/phototracker.cpp": ["bool PhotoTracker::poseDifferenceExceeded"],
}


def strip_comments(src: str) -> str:
    src = re.sub(r"/\*.*?\*/", lambda m: "\n" * m.group(0).count("\n"), src, flags=re.S)
    return re.sub(r"//[^\n]*", "", src)


def extract(src: str, name: str) -> str:
    if " " in name:  # a full declarator prefix, e.g. "bool Class::method"
        m = re.search(re.escape(name) + r"\s*\(", src)
    else:
        m = re.search(r"(__global__|__device__)[^;{()]*?\b" + re.escape(name) + r"\s*\(", src)
    if not m:
        raise RuntimeError(f"function {name} not found")
    start = m.start()
    i = src.index("{", m.end())
    depth = 0
    for j in range(i, len(src)):
        if src[j] == "{":
            depth += 1
        elif src[j] == "}":
            depth -= 1
            if depth == 0:
                return src[start:j + 1] + "\n"
    raise RuntimeError(f"unbalanced braces in {name}")


def main() -> int:
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("RECON_REFERENCE", "")
    if not ref or not os.path.isdir(os.path.join(ref, "tracker", "kernels")):
        print(f"reference tree not found ({ref or 'no path given'}); oracle/_ref not built")
        return 1
    os.makedirs(OUT, exist_ok=True)
    for rel, names in FRAGMENTS.items():
        with open(os.path.join(ref, rel), encoding="latin-1") as f:
            src = strip_comments(f.read())
        body = "".join(extract(src, n) for n in names)
        base = os.path.splitext(os.path.basename(rel))[0]
        with open(os.path.join(OUT, f"frag_{base}.inc"), "w") as f:
            f.write(f"// extracted from {rel}: {', '.join(names)}\n" + body)
    # particles_kernel.cuh includes the CUDA header vector_types.h; the shim
    # defines the vector types itself, so an empty stand-in satisfies it
    stub = os.path.join(OUT, "stub")
    os.makedirs(stub, exist_ok=True)
    with open(os.path.join(stub, "vector_types.h"), "w") as f:
        f.write("// empty: the vector types come from ref_shim.cpp\n")
    # TrackingParams.h includes tracker/phototracker.h (CUDA headers) for the
    # TrackMode enum alone; the stand-in declares that enum
    os.makedirs(os.path.join(stub, "tracker"), exist_ok=True)
    with open(os.path.join(stub, "tracker", "phototracker.h"), "w") as f:
        f.write("#pragma once\nenum TrackMode { GEOMETRIC, PHOTOMETRIC, BIOBJECTIVE };\n")
    cxx = os.environ.get("CXX", "g++")
    flags = ["-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-w", "-std=c++20", "-pthread"]
    inc = ["-I" + OUT, "-I" + stub, "-I" + os.path.join(ref, "tracker"), "-I" + os.path.join(ref, "tracker", "kernels"),
           "-I" + os.path.join(ref, "tracker", "tracker")]
    objs = []
    shim_o = os.path.join(OUT, "ref_shim.o")
    subprocess.run([cxx, *flags, *inc, "-c", os.path.join(HERE, "ref_shim.cpp"), "-o", shim_o], check=True)
    objs.append(shim_o)
    expm_o = os.path.join(OUT, "expm.o")
    subprocess.run([cxx, *flags, *inc, "-x", "c++", "-include", "cmath", "-include", "cstdio", "-c",
                    os.path.join(ref, "tracker", "tracker", "expm.c"), "-o", expm_o], check=True)
    objs.append(expm_o)
    bm_o = os.path.join(OUT, "basic_math.o")
    subprocess.run([cxx, *flags, *inc, "-c", os.path.join(ref, "tracker", "tracker", "basic_math.cpp"), "-o", bm_o],
                   check=True)
    objs.append(bm_o)
    # the result files (ResultTxt and TrackingParams as they are) and the
    # wrappers of the result files and of the Kinect routines
    for src, obj in ((os.path.join(ref, "tracker", "calib", "ResultTxt.cpp"), "ResultTxt.o"),
                     (os.path.join(ref, "tracker", "calib", "TrackingParams.cpp"), "TrackingParams.o"),
                     (os.path.join(HERE, "ref_files.cpp"), "ref_files.o"),
                     (os.path.join(HERE, "ref_multicore.cpp"), "ref_multicore.o")):
        o = os.path.join(OUT, obj)
        subprocess.run([cxx, *flags, *inc, "-c", src, "-o", o], check=True)
        objs.append(o)
    subprocess.run([cxx, "-shared", "-pthread", "-o", os.path.join(OUT, "libreconref.so"), *objs], check=True)
    print("built", os.path.join(OUT, "libreconref.so"))
    return 0


if __name__ == "__main__":
    sys.exit(main())
