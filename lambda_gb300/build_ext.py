"""Build recipe of the CUDA extension: nvcc for sm_103a, in-tree output (lambda_gb300/_build/).

Each translation unit compiles in parallel; the shared library exports only the C ABI of
include/lambda_gpu.h.  Host code is compiled with -ffp-contract=off so the light-tree build and
other host arithmetic are identical on x86 and Arm hosts.
"""
import concurrent.futures as cf
import os
import pathlib
import shutil
import subprocess

HERE = pathlib.Path(__file__).resolve().parent
CSRC = HERE / "csrc"
OUT = HERE / "_build"
LIB = OUT / "liblambda_gpu.so"
# (source, extra defines, object name); the render megakernel is built once per variant
# Render kernels: one unit per (spectral mode, counter variant, part); part 1 MIS megakernel, 2 wavefront
# resume/spawn, 3 trace + closest-hit batches + film kernels (RGB3 only), 4 adjoint (RGB3, no counters),
# 5 megakernel of the other integrators.
_PARTS = [(ns, cnt, part) for ns in (3, 4) for cnt in (0, 1) for part in (1, 2, 3, 4, 5)
          if (part != 3 or ns == 3) and (part != 4 or (ns == 3 and cnt == 0))]
SOURCES = [("lgpu_api.cu", [], "lgpu_api"), ("lgpu_compile.cu", [], "lgpu_compile"),
           ("lgpu_lighttree.cpp", [], "lgpu_lighttree"), ("lgpu_lbvh.cu", [], "lgpu_lbvh")] + [
    ("lgpu_render.cu", ["-DLGPU_NS=%d" % ns, "-DLGPU_COUNT=%d" % cnt, "-DLGPU_PART=%d" % part],
     "render_%d_%d_p%d" % (ns, cnt, part)) for ns, cnt, part in _PARTS]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return p


def _flags(fmad=False):
    """Device code is compiled without multiply-add contraction (-fmad=false), as the host code and the
    CPU checkers are (-ffp-contract=off): every a * b + c rounds twice, as in the reference, so a
    path's sampling decisions are the reference's own.  With contraction, 2-3 % of the paths of the
    full-size scenes took another branch on a last-bit difference."""
    return ["-O3", "-std=c++17", "-lineinfo", *ARCH, "-fmad=%s" % ("true" if fmad else "false"),
            "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden",
            "-I" + str(CSRC), "-I" + str(HERE.parent / "include")]


def build(force=False, verbose=False, defines=(), out_dir=None, extra_flags=(), fmad=False):
    """Compile into lambda_gb300/_build (or out_dir, for variants built with extra -D defines such
    as LGPU_RESUME_MINB=5 or LGPU_NO_STAGE, extra nvcc flags, or fmad=True for contraction)."""
    out = pathlib.Path(out_dir) if out_dir else OUT
    lib_path = out / LIB.name
    out.mkdir(parents=True, exist_ok=True)
    deps = list(CSRC.glob("*")) + [HERE.parent / "include" / "lambda_gpu.h", pathlib.Path(__file__)]
    newest = max(p.stat().st_mtime for p in deps)
    if lib_path.exists() and not force and lib_path.stat().st_mtime >= newest:
        return lib_path

    def compile_one(spec):
        src, defs, name = spec
        obj = out / (name + ".o")
        cmd = [nvcc(), *_flags(fmad), *defs, *["-D" + d for d in defines], *extra_flags, "-c", str(CSRC / src), "-o", str(obj)]
        if verbose and src.endswith(".cu"):
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed on %s:\n%s\n%s" % (src, r.stdout, r.stderr))
        return obj, r.stderr

    # the slowest units first (resume/spawn, the other integrators, the adjoint, the MIS megakernel),
    # so the pool's last jobs are short ones
    rank = {"-DLGPU_PART=2": 0, "-DLGPU_PART=5": 1, "-DLGPU_PART=4": 2, "-DLGPU_PART=1": 3}
    order = sorted(SOURCES, key=lambda sp: min([rank.get(d, 9) for d in sp[1]] + [9]))
    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 8)) as ex:
        results = list(ex.map(compile_one, order))
    objs = [str(o) for o, _ in results]
    if verbose:
        for _, log in results:
            print(log)
    tmp = lib_path.with_suffix(".so.tmp%d" % os.getpid())
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, lib_path)
    return lib_path


if __name__ == "__main__":
    import sys
    print(build(force="-f" in sys.argv, verbose="-v" in sys.argv))
