"""Build recipe for oracle/_ref/libyvref.so: the reference's own renderer
code compiled on the host, from where it lies in the reference checkout,
to pin the oracle (test infrastructure only; nothing of the product links
or loads it).

Compiled sources of the reference (znah/yoxel-voxel):
  cell/ppu_renderer.cpp      the CPU renderer: RecTrace, RenderRect,
                             SimpleRenderer / TreadedRenderer, with
                             cell/renderer_base.h (InitRayDir), svorenderer.h,
                             svodata.h (SVOData::Load), alignedarray.h
  cell/spu/trace_spu.cpp     the SPU tracer: FindFirstChildSPU, GoNextSPU,
                             RecTrace, FetchNode, RenderBlock
  reaction/trace/trace.cu    the brick-skipping volume march: castRay,
                             walkBrick, intersect (with its utils.h)
The headers their snapshot lacks (cpp/, Boost, the Cell SDK, CUDA) are
stood in for by oracle/ref_shim/.  Outputs go to oracle/_ref/ only.

Without the reference checkout (REFERENCE_ROOT, default the checkout next
to this repository's build container) nothing is built and the tests that
use the library skip.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
OUT = os.path.join(OUT_DIR, "libyvref.so")
SHIM = os.path.join(HERE, "ref_shim")


def reference_root():
    return os.environ.get("REFERENCE_ROOT", "/root/reference")


def available():
    r = reference_root()
    return all(os.path.exists(os.path.join(r, p)) for p in
               ("cell/ppu_renderer.cpp", "cell/spu/trace_spu.cpp", "reaction/trace/trace.cu"))


def _units(ref):
    common = ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-w",
              "-pthread", "-I" + SHIM]
    return [
        (common + ["-fpermissive", "-Dmain=yvref_spu_main", "-DTraceResult=YvrefSpuTraceResult",
                   "-I" + os.path.join(ref, "cell", "spu"),
                   os.path.join(HERE, "ref_spu_glue.cpp")], "spu.o"),
        (common + [os.path.join(ref, "cell", "ppu_renderer.cpp")], "ppu.o"),
        (common + ["-I" + os.path.join(ref, "cell"), os.path.join(HERE, "ref_harness.cpp")],
         "harness.o"),
        (common + ["-I" + os.path.join(ref, "reaction", "trace"),
                   os.path.join(HERE, "ref_march_glue.cpp")], "march.o"),
    ]


def build(force=False, verbose=False):
    """Compile oracle/_ref/libyvref.so if the reference checkout is present.
    Returns its path, or None when the reference is absent."""
    if not available():
        return None
    os.makedirs(OUT_DIR, exist_ok=True)
    deps = [os.path.join(SHIM, f) for f in os.listdir(SHIM) if f.endswith(".h")]
    deps += [os.path.join(HERE, f) for f in ("ref_spu_glue.cpp", "ref_harness.cpp",
                                             "ref_march_glue.cpp", "build_ref.py")]
    if not force and os.path.exists(OUT):
        t = os.path.getmtime(OUT)
        if all(os.path.getmtime(d) <= t for d in deps):
            return OUT
    units = _units(reference_root())
    objs = []
    with cf.ThreadPoolExecutor(max_workers=len(units)) as ex:
        futs = []
        for cmd, obj in units:
            o = os.path.join(OUT_DIR, obj)
            objs.append(o)
            full = cmd + ["-c", "-o", o]
            if verbose:
                print(" ".join(full))
            futs.append(ex.submit(subprocess.run, full, capture_output=True, text=True))
        errs = [f.result() for f in futs if f.result().returncode != 0]
    if errs:
        raise RuntimeError("reference build failed:\n" + "\n".join(e.stderr for e in errs))
    cmd = ["g++", "-shared", "-pthread", "-o", OUT + ".tmp"] + objs
    subprocess.run(cmd, check=True)
    os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
