"""In-tree build of the engine's native libraries (no cmake, no torch).

``build_all()`` compiles, in parallel:

* ``lib/libhbt_gpu.so`` - the CUDA kernels and the C ABI (include/hbt_gpu.h),
  for sm_103a only;
* ``lib/libhbt_host.so`` and ``lib/hbt_afterburner.e`` - the C++ drop-in host
  side (parameter reader, event reader, HBT_correlation driver, writer),
  when its sources are present;
* ``oracle/liboracle.so`` - the CPU oracle the tests compare against.

The pair-binning translation unit is compiled with ``--fmad=false`` so that
no FP64 multiply-add is contracted: every bin-deciding operation rounds as
the reference's CPU build does.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
LIB = os.path.join(PKG, "lib")
OBJ = os.path.join(PKG, "lib", "obj")
INCLUDE = os.path.join(REPO, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                      "-Xcompiler", "-ffp-contract=off", "-I" + INCLUDE, "-I" + CSRC]

# translation unit -> extra flags
GPU_UNITS = {
    "hbt_kernels.cu": ["--fmad=false"],
    "hbt_capi.cu": ["--fmad=false"],
    "hbt_fast.cu": ["--fmad=false"],
    "hbt_noalloc.cu": ["--fmad=false"],
    "hbt_batch.cu": ["--fmad=false"],
    "hbt_persist_fast.cu": ["--fmad=false"],
    "hbt_persist_caps.cu": ["--fmad=false"],
    "hbt_persist_qinv.cu": ["--fmad=false"],
    "hbt_runner.cu": [],
    "hbt_server.cu": ["--fmad=false"],
    "hbt_bf.cu": ["--fmad=false"],
    "hbt_fit.cu": [],
    "hbt_check.cu": ["--fmad=false"],
}


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd, cwd=None):
    proc = subprocess.run(cmd, cwd=cwd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s%s" % (" ".join(cmd), proc.stdout, proc.stderr))
    return proc.stdout + proc.stderr


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _gpu_deps():
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    return deps


def build_gpu(force: bool = False, verbose: bool = False) -> str:
    """Compile libhbt_gpu.so; returns its path."""
    os.makedirs(OBJ, exist_ok=True)
    out = os.path.join(LIB, "libhbt_gpu.so")
    deps = _gpu_deps()
    if not force and not _newer(out, deps):
        return out
    nvcc = _nvcc()
    objs = []
    jobs = []
    with cf.ThreadPoolExecutor(max_workers=len(GPU_UNITS)) as ex:
        for unit, extra in GPU_UNITS.items():
            obj = os.path.join(OBJ, unit.replace(".cu", ".o"))
            objs.append(obj)
            defines = os.environ.get("HBT_NVCC_DEFINES", "").split()
            cmd = [nvcc] + NVCC_COMMON + extra + defines + ["-Xptxas", "-v", "-c",
                                                  os.path.join(CSRC, unit), "-o", obj]
            jobs.append(ex.submit(_run, cmd))
        logs = [j.result() for j in jobs]
    if verbose:
        for log in logs:
            sys.stdout.write(log)
    _run([nvcc] + ARCH + ["-shared", "-o", out] + objs)
    return out


def build_probe(force: bool = False) -> str:
    """libhbt_probe.so: FP64 / FP32 pipe-throughput probes for the bench."""
    os.makedirs(LIB, exist_ok=True)
    src = os.path.join(CSRC, "hbt_probe.cu")
    out = os.path.join(LIB, "libhbt_probe.so")
    if force or _newer(out, [src]):
        _run([_nvcc()] + ARCH + ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
                                 src, "-o", out])
    return out


def build_host(force: bool = False) -> str | None:
    """Compile the C++ drop-in host library and CLI if their sources exist."""
    srcs = sorted(os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".cpp")) \
        if os.path.isdir(HOST) else []
    if not srcs:
        return None
    os.makedirs(LIB, exist_ok=True)
    gpu = build_gpu(force=False)
    lib = os.path.join(LIB, "libhbt_host.so")
    exe = os.path.join(LIB, "hbt_afterburner.e")
    deps = srcs + [os.path.join(HOST, f) for f in os.listdir(HOST)] + [gpu]
    if force or _newer(lib, deps) or _newer(exe, deps):
        cxx = os.environ.get("CXX", "g++")
        flags = ["-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-pthread",
                 "-I" + INCLUDE, "-I" + HOST]
        zlib = _has_zlib(cxx)
        if zlib:
            flags.append("-DHBT_HAVE_ZLIB=1")
        libs = ["-L" + LIB, "-lhbt_gpu", "-Wl,-rpath,$ORIGIN"] + (["-lz"] if zlib else [])
        lib_srcs = [s for s in srcs if not s.endswith("main.cpp")]
        _run([cxx] + flags + ["-shared", "-o", lib] + lib_srcs + libs)
        # one executable per *main.cpp: main.cpp -> hbt_afterburner.e,
        # average_main.cpp -> hbt_average.e
        for m in (s for s in srcs if s.endswith("main.cpp")):
            base = os.path.basename(m)
            out = exe if base == "main.cpp" else os.path.join(
                LIB, "hbt_" + base[:-len("_main.cpp")] + ".e")
            _run([cxx] + flags + ["-o", out, m, "-L" + LIB, "-lhbt_host", "-lhbt_gpu",
                                  "-Wl,-rpath,$ORIGIN"])
    return lib


def _has_zlib(cxx: str) -> bool:
    probe = os.path.join(OBJ, "zprobe.cpp")
    os.makedirs(OBJ, exist_ok=True)
    with open(probe, "w") as f:
        f.write("#include <zlib.h>\nint main(){gzFile f=gzopen(\"x\",\"rb\");return f?0:1;}\n")
    proc = subprocess.run([cxx, probe, "-o", probe + ".out", "-lz"], capture_output=True)
    return proc.returncode == 0


def build_oracle() -> str:
    _run(["make", "-s", "-C", os.path.join(REPO, "oracle")])
    return os.path.join(REPO, "oracle", "liboracle.so")


def build_reference(ref_root: str | None = None) -> str | None:
    """Compile the unmodified reference into oracle/_ref when a checkout of
    it is found: ``ref_root``, else the one oracle/Makefile finds (the
    environment variable HBT_REFERENCE_ROOT, else where the checkout is
    mounted on the development machine).  None when there is none."""
    target = ["ref", "REF=" + ref_root] if ref_root else ["ref-if-present"]
    if ref_root and not os.path.isdir(os.path.join(ref_root, "src")):
        return None
    try:
        _run(["make", "-s", "-C", os.path.join(REPO, "oracle")] + target)
    except RuntimeError:
        return None
    exe = os.path.join(REPO, "oracle", "_ref", "hadronic_afterburner_tools.e")
    return exe if os.path.exists(exe) else None


def build_all(force: bool = False, verbose: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=4) as ex:
        f_gpu = ex.submit(build_gpu, force, verbose)
        f_prb = ex.submit(build_probe, force)
        f_orc = ex.submit(build_oracle)
        f_ref = ex.submit(build_reference)
        f_gpu.result()
        f_prb.result()
        f_orc.result()
        f_ref.result()
    build_host(force)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv, verbose=True)
