"""In-tree build of the GB300 library (CUDA for sm_103a) and of the test-only
CPU oracle.

    python -m fvens_gb300.build            # library + oracle (+ reference shim when present)

Outputs (git-ignored):
    fvens_gb300/lib/libfvens_gb300.so      the product: C ABI in include/fvens_gb300.h
    oracle/build/liborc.so                 CPU restatement used only by tests and the CPU baseline
    oracle/_ref/libfvens_ref.so            reference pointwise physics (only where the reference is present)
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
OBJDIR = os.path.join(HERE, "lib", "obj")
LIB = os.path.join(LIBDIR, "libfvens_gb300.so")
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "build", "liborc.so")
REF_LIB = os.path.join(ORACLE_DIR, "_ref", "libfvens_ref.so")

NVCC_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-O3", "-std=c++17", "-lineinfo",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
    "--expt-relaxed-constexpr",
    "-diag-suppress", "177,1444",
]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".hpp", ".h"))]
    hs.append(os.path.join(ROOT, "include", "fvens_gb300.h"))
    return hs


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def build_library(verbose=False, jobs=None):
    os.makedirs(OBJDIR, exist_ok=True)
    nvcc = _nvcc()
    srcs = sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))
    hdrs = _headers()
    cmds, objs = [], []
    for s in srcs:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OBJDIR, s + ".o")
        objs.append(obj)
        if _stale(obj, [src] + hdrs):
            if s.endswith(".cu"):
                cmds.append([nvcc] + NVCC_FLAGS + ["-c", src, "-o", obj])
            else:
                cmds.append(["g++", "-std=c++17", "-O2", "-fPIC", "-Wall", "-c", src, "-o", obj])
    if cmds:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(len(cmds), os.cpu_count() or 4)) as ex:
            for out in ex.map(_run, cmds):
                if verbose and out.strip():
                    print(out)
    if _stale(LIB, objs):
        _run([nvcc, "-shared", "-gencode", "arch=compute_103a,code=sm_103a", "-o", LIB] + objs + ["-lcudart"])
    return LIB


def build_oracle():
    os.makedirs(os.path.dirname(ORACLE_LIB), exist_ok=True)
    srcs = [os.path.join(ORACLE_DIR, f) for f in ("orc_core.cpp", "orc_physics.hpp", "orc_dual.hpp")]
    if _stale(ORACLE_LIB, srcs):
        _run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-Wall",
              os.path.join(ORACLE_DIR, "orc_core.cpp"), "-o", ORACLE_LIB])
    return ORACLE_LIB


def build_reference_shim(reference_root=None):
    """Compiles the reference's own pointwise physics into oracle/_ref (only
    where the reference sources exist).  reference_root: the reference
    project's root; by default oracle/ref/build_ref.sh picks it
    ($FVENS_REFERENCE or its own default) and skips when it is absent."""
    shim = os.path.join(ORACLE_DIR, "ref", "ref_wrap.cpp")
    recipe = os.path.join(ORACLE_DIR, "ref", "build_ref.sh")
    if _stale(REF_LIB, [shim, recipe]):
        _run(["sh", recipe] + ([reference_root] if reference_root else []))
    return REF_LIB if os.path.exists(REF_LIB) else None


def build_all(verbose=False):
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        f_lib = ex.submit(build_library, verbose)
        f_orc = ex.submit(build_oracle)
        lib, orc = f_lib.result(), f_orc.result()
    ref = build_reference_shim()
    return lib, orc, ref


if __name__ == "__main__":
    out = build_all(verbose="-v" in sys.argv)
    for p in out:
        if p:
            print("built", p)
