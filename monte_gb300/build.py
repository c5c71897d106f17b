"""Build libmonte.so in-tree for sm_103a (no torch extension machinery).

    python -m monte_gb300.build            # or monte_gb300.build.build()

Every .cu/.cpp under csrc/ is compiled to an object in parallel with nvcc
(-gencode arch=compute_103a,code=sm_103a), then linked into
monte_gb300/libmonte.so.  The host programs under programs/ are linked
against it.  Objects go to monte_gb300/_build/ (git-ignored).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmonte.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc")

# -fmad=false: the Monte Carlo kernels must round exactly like the host
# replay harness, the tiled backprojector's tile shapes must give the same
# volumes bit for bit, and the double-precision restatements (fbp2, the
# exact decisions) follow the reference's operation order; their fused
# multiply-adds are written explicitly as fmaf().  The files in FMAD_ON
# compare with the oracle within a tolerance only, and let the compiler
# fuse multiply-adds (their float-pair arithmetic uses the _rn intrinsics,
# which are never fused).
CU_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
            "--prec-div=true", "--prec-sqrt=true", "-Xptxas", "-warn-spills",
            "--expt-relaxed-constexpr"]
FMAD_ON = {"fdk_adjoint.cu", "fdk_filter_fp32.cu", "fdk_filter_bf16x3.cu", "fdk_bp_plain.cu"}
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall",
             "-I/usr/local/cuda/include"]


def _newer(src, obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + deps)


def _compile(src, deps):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if not _newer(src, obj, deps):
        return obj, None
    if src.endswith(".cu"):
        fmad = "-fmad=true" if os.path.basename(src) in FMAD_ON else "-fmad=false"
        cmd = [NVCC] + ARCH + CU_FLAGS + [fmad, "-c", src, "-o", obj]
    else:
        cmd = ["g++"] + CXX_FLAGS + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return obj, "FAILED: " + " ".join(cmd) + "\n" + r.stdout + r.stderr
    return obj, (r.stdout + r.stderr).strip() or None


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)
                  if f.endswith((".cu", ".cpp")))
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    deps.append(os.path.join(os.path.dirname(HERE), "include", "monte.h"))
    deps.append(os.path.abspath(__file__))  # compile flags
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        results = list(ex.map(lambda s: _compile(s, deps), srcs))
    errs = [m for _, m in results if m and m.startswith("FAILED")]
    if errs:
        raise RuntimeError("\n".join(errs))
    if verbose:
        for o, m in results:
            if m:
                print(os.path.basename(o), m)
    objs = [o for o, _ in results]
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart_static", "-lrt", "-ldl",
                                                             "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    _build_programs()
    return LIB


def _build_programs():
    pdir = os.path.join(HERE, "programs")
    if not os.path.isdir(pdir):
        return
    for f in sorted(os.listdir(pdir)):
        if not f.endswith(".cpp"):
            continue
        exe = os.path.join(pdir, f[:-4])
        src = os.path.join(pdir, f)
        if os.path.exists(exe) and os.path.getmtime(exe) > max(os.path.getmtime(src),
                                                               os.path.getmtime(LIB)):
            continue
        cmd = ["g++", "-O2", "-std=c++17", "-o", exe, src, "-I" + os.path.dirname(HERE),
               "-L" + HERE, "-lmonte", "-Wl,-rpath,$ORIGIN/.."]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("program build failed: " + " ".join(cmd) + "\n" + r.stderr)


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
