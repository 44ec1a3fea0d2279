"""Builds oracle/_ref/libpsim_ref.so: the reference's own hot-path sources,
compiled where they lie under /root/reference with g++ -fopenmp and the
Thrust OpenMP back end of the CUDA toolkit, plus the shims and the harness in
oracle/ref_harness.  TEST INFRASTRUCTURE ONLY (checker); the product never
links it.  Nothing is copied from the reference tree; outputs go to
oracle/_ref only.  Returns None when the reference tree is absent.
"""
import glob
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("PANSIM_REFERENCE", "/root/reference")
OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT, "libpsim_ref.so")

# reference translation units on the hot path
REF_SOURCES = [
    "src/tools/timeDay.cpp", "src/tools/operators.cpp", "src/tools/timeHandler.cpp", "src/tools/smallTools.cpp",
    "src/tools/util.cpp", "src/tools/timing.cpp",
    "src/tools/progressionMatrices/multiBadMatrix.cpp", "src/tools/progressionMatrices/basicLengthAbstract.cpp",
    "src/agentData/dynamicPPState.cpp", "src/agentData/agentMeta.cpp", "src/agentData/agentType.cpp",
    "src/agentData/globalStates.cpp", "src/agentData/agentStat.cpp", "src/IO/dataProviders/progressionType.cpp",
]
# sources that need shim/thrust_compat.h (by-value make_pair / make_tuple)
COMPAT_SOURCES = {"multiBadMatrix.cpp"}
REF_INCLUDES = ["include", "include/tools", "include/tools/progressionMatrices", "include/agentData",
                "include/policies", "include/IO", "include/IO/inputFormats", "include/IO/dataProviders",
                "include/IO/outputs"]


def cccl_include():
    cands = glob.glob("/usr/local/cuda/targets/*/include/cccl") + glob.glob("/usr/local/cuda/include/cccl")
    for c in cands:
        if os.path.isdir(os.path.join(c, "thrust")):
            return c
    raise RuntimeError("CCCL (Thrust) headers not found in the CUDA toolkit")


def available():
    return os.path.isdir(os.path.join(REF, "include", "policies"))


def flags():
    inc = ["-I", os.path.join(HERE, "ref_harness", "shim")]
    for d in REF_INCLUDES:
        inc += ["-I", os.path.join(REF, d)]
    inc += ["-I", cccl_include()]
    return ["g++", "-std=c++17", "-O2", "-fopenmp", "-fPIC", "-ffp-contract=off", "-w",
            "-DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_OMP", "-DTHRUST_HOST_SYSTEM=THRUST_HOST_SYSTEM_CPP",
            "-D__host__=", "-D__device__=", "-include", "cstdint"] + inc


def build(force=False, verbose=False):
    if not available():
        return None
    os.makedirs(OUT, exist_ok=True)
    srcs = [os.path.join(REF, s) for s in REF_SOURCES] + [os.path.join(HERE, "ref_harness", "harness.cpp")]
    deps = srcs + glob.glob(os.path.join(HERE, "ref_harness", "shim", "*")) + [
        os.path.join(HERE, "..", "pansim_gb300", "csrc", "psim_rng.h"), os.path.join(HERE, "..", "include", "pansim_gb300.h")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    objs, jobs = [], []
    compat = ["-include", os.path.join(HERE, "ref_harness", "shim", "thrust_compat.h")]
    for s in srcs:
        o = os.path.join(OUT, os.path.basename(s).replace(".cpp", ".o"))
        objs.append(o)
        extra = compat if os.path.basename(s) in COMPAT_SOURCES else []
        jobs.append(flags() + extra + ["-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        res = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
    for cmd, r in zip(jobs, res):
        if r.returncode or verbose:
            sys.stderr.write(r.stdout + r.stderr[-6000:])
        if r.returncode:
            raise RuntimeError("compile failed: " + cmd[-3])
    tmp = LIB + ".%d.tmp" % os.getpid()
    subprocess.check_call(["g++", "-shared", "-fopenmp", "-o", tmp] + objs)
    os.replace(tmp, LIB)
    return LIB


def check_adapters():
    """Compiles (syntax only) oracle/ref_harness/adapter_check.cpp: the
    reference's own Simulation instantiated with the GB300 policies of
    include/gb300_policies.h.  Returns (ok, compiler output), or None when
    the reference tree is absent."""
    if not available():
        return None
    src = os.path.join(HERE, "ref_harness", "adapter_check.cpp")
    cmd = flags() + ["-I", os.path.join(HERE, "..", "include"), "-fsyntax-only", src]
    r = subprocess.run(cmd, capture_output=True, text=True)
    return r.returncode == 0, r.stderr[-8000:]


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
