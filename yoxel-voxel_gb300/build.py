"""Builds the yoxel GB300 library: libyoxel.so (CUDA kernels + C ABI).

Every translation unit in csrc/ is compiled in parallel (.cu with nvcc for
sm_103a, .cpp with g++), then linked with nvcc into yoxel/libyoxel.so next to
the Python binding.  No cmake; one -gencode.  Host code is compiled with
-ffp-contract=off (one IEEE rounding per written float operation) and
without target-specific flags, so it builds and behaves the same on x86_64
and aarch64.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INC = os.path.join(ROOT, "include")
OBJ = os.path.join(HERE, "_build")
OUT = os.path.join(HERE, "yoxel", "libyoxel.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else (shutil.which("nvcc") or "nvcc")


def _cuda_inc():
    return os.path.join(os.path.dirname(os.path.dirname(_nvcc())), "include")


def _sources():
    srcs = []
    for f in sorted(os.listdir(CSRC)):
        if f.endswith((".cu", ".cpp")):
            srcs.append(os.path.join(CSRC, f))
    return srcs


def _headers():
    hs = [os.path.join(INC, f) for f in os.listdir(INC) if f.endswith(".h")]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs


def _compile_cmd(src, obj):
    common = ["-I" + INC, "-I" + CSRC]
    if src.endswith(".cu"):
        return [_nvcc(), "-std=c++17", "-O3", "-lineinfo", *ARCH, *common,
                "-Xcompiler", "-fPIC,-ffp-contract=off", "-c", src, "-o", obj]
    return ["g++", "-std=c++17", "-O3", "-fPIC", "-ffp-contract=off", "-pthread",
            "-Wall", "-Wno-unused-function", *common, "-I" + _cuda_inc(),
            "-c", src, "-o", obj]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, jobs=None):
    """Compile and link libyoxel.so if any source is newer.  Returns its path."""
    os.makedirs(OBJ, exist_ok=True)
    srcs = _sources()
    hdrs = _headers()
    objs, todo = [], []
    for s in srcs:
        o = os.path.join(OBJ, os.path.basename(s) + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            todo.append((s, o))
    if todo:
        jobs = jobs or min(len(todo), os.cpu_count() or 4)
        with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
            futs = {}
            for s, o in todo:
                cmd = _compile_cmd(s, o)
                if verbose:
                    print(" ".join(cmd), flush=True)
                futs[ex.submit(subprocess.run, cmd, capture_output=True, text=True)] = s
            errs = []
            for f in cf.as_completed(futs):
                r = f.result()
                if r.returncode != 0:
                    errs.append(f"{futs[f]}:\n{r.stdout}{r.stderr}")
                elif verbose and (r.stdout or r.stderr):
                    print(r.stdout + r.stderr, flush=True)
            if errs:
                raise RuntimeError("yoxel build failed:\n" + "\n".join(errs))
    if force or todo or _stale(OUT, objs):
        cmd = [_nvcc(), "-shared", *ARCH, "-o", OUT + ".tmp", *objs,
               "-cudart", "static", "-lpthread", "-ldl", "-lrt"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("yoxel link failed:\n" + r.stdout + r.stderr)
        os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
