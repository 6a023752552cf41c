"""Build recipe for the CPU oracle (TEST INFRASTRUCTURE ONLY).

* ``build_oracle()`` compiles the project's C restatement ``mf_oracle.c`` into
  ``oracle/liborc.so`` (OpenMP, portable flags: it is built on the x86 dev
  host and on the Arm GPU host alike).
* ``build_ref()`` compiles the reference mflib sources *unchanged*, from where
  they lie in the read-only reference checkout, against the project-written
  FFTW/MKL shim in ``oracle/ref_shim/``, together with ``ref_driver.cpp``, into
  ``oracle/_ref/libmflib_ref.so``.  It is skipped when the reference checkout
  is absent.  Nothing is copied out of the reference tree.

Run ``python oracle/build.py`` to build both.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# Where this recipe reads the reference checkout: $MFLIB_REFERENCE_ROOT (the
# repository's build() sets it when the development host's checkout exists).
# Without it build_ref() is skipped and the tests that need the compiled
# reference skip with it.


def ref_root():
    return os.environ.get("MFLIB_REFERENCE_ROOT") or ""
REF_SOURCES = [
    "src/matchedFilter.cpp",
    "src/matchedFilterParameters.cpp",
    "src/waveformTemplate.cpp",
    "src/networkStationPhase.cpp",
    "src/peakFinder.cpp",
    "src/singleChannel/matchedFilter.cpp",
    "src/singleChannel/matchedFilterParameters.cpp",
    "src/singleChannel/detector.cpp",
    "src/singleChannel/detectorParameters.cpp",
    "src/singleChannel/detectionTimeInterpolationParameters.cpp",
    "src/singleChannel/detection.cpp",
    "src/singleChannel/relativeMagnitude.cpp",
]


def _run(cmd):
    subprocess.run(cmd, check=True)


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def oracle_lib_path():
    return os.path.join(HERE, "liborc.so")


def ref_lib_path():
    return os.path.join(HERE, "_ref", "libmflib_ref.so")


def build_oracle(force=False):
    out = oracle_lib_path()
    deps = [os.path.join(HERE, f) for f in ("mf_oracle.c", "orc_fft.h", "orc_mf.h")]
    if force or _stale(out, deps):
        _run(["gcc", "-std=c11", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-fopenmp",
              "-fvisibility=hidden", "-o", out, deps[0], "-lm"])
    return out


def build_ref(force=False):
    REF_ROOT = ref_root()
    if not REF_ROOT or not os.path.isdir(os.path.join(REF_ROOT, "src")):
        return None
    outdir = os.path.join(HERE, "_ref")
    os.makedirs(outdir, exist_ok=True)
    out = ref_lib_path()
    srcs = [os.path.join(REF_ROOT, s) for s in REF_SOURCES]
    deps = srcs + [os.path.join(HERE, "ref_driver.cpp"),
                   os.path.join(HERE, "ref_shim", "shim.c"),
                   os.path.join(HERE, "orc_fft.h")]
    if not (force or _stale(out, deps)):
        return out
    objs = []
    shim_obj = os.path.join(outdir, "shim.o")
    _run(["gcc", "-std=c11", "-O2", "-fPIC", "-c", "-o", shim_obj,
          os.path.join(HERE, "ref_shim", "shim.c")])
    objs.append(shim_obj)
    inc = ["-I", os.path.join(HERE, "ref_shim"), "-I", os.path.join(REF_ROOT, "include")]
    # HAVE_STD__MAKE_UNIQUE is what the reference's own CMake defines after
    # its configure probe; without it include/private/private.hpp does not
    # compile.
    cxx = ["g++", "-std=c++17", "-O2", "-fPIC", "-fopenmp", "-DHAVE_STD__MAKE_UNIQUE=1",
           "-w"] + inc
    for s in srcs + [os.path.join(HERE, "ref_driver.cpp")]:
        o = os.path.join(outdir, os.path.basename(os.path.dirname(s)) + "_"
                         + os.path.splitext(os.path.basename(s))[0] + ".o")
        flags = cxx
        if s.endswith(os.path.join("singleChannel", "detector.cpp")):
            # its "omp simd aligned(mfPtr: 64)" clauses (reduceAllCorrelations,
            # src/singleChannel/detector.cpp:212, :230) promise 64-byte
            # alignment of trace pointers that start at L - 1; with OpenMP
            # SIMD on, the absolute-maximum reduction faults.  Compiled
            # without OpenMP the pragmas are ignored and the code is the same.
            flags = [f for f in cxx if f != "-fopenmp"]
        _run(flags + ["-c", "-o", o, s])
        objs.append(o)
    _run(["g++", "-shared", "-fopenmp", "-o", out] + objs + ["-lm"])
    for o in objs:
        os.remove(o)
    return out


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
