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
SOURCES = [("lgpu_api.cu", [], "lgpu_api"), ("lgpu_compile.cu", [], "lgpu_compile"),
           ("lgpu_lighttree.cpp", [], "lgpu_lighttree"),
           ("lgpu_render.cu", ["-DLGPU_NS=3", "-DLGPU_COUNT=0"], "render_3_0"),
           ("lgpu_render.cu", ["-DLGPU_NS=3", "-DLGPU_COUNT=1"], "render_3_1"),
           ("lgpu_render.cu", ["-DLGPU_NS=4", "-DLGPU_COUNT=0"], "render_4_0"),
           ("lgpu_render.cu", ["-DLGPU_NS=4", "-DLGPU_COUNT=1"], "render_4_1")]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return p


def _flags():
    return ["-O3", "-std=c++17", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden",
            "-I" + str(CSRC), "-I" + str(HERE.parent / "include")]


def build(force=False, verbose=False, defines=(), out_dir=None):
    """Compile into lambda_gb300/_build (or out_dir, for tuning variants built with extra
    -D defines such as LGPU_RESUME_MINB=5 or LGPU_NO_STAGE)."""
    out = pathlib.Path(out_dir) if out_dir else OUT
    lib_path = out / LIB.name
    out.mkdir(parents=True, exist_ok=True)
    deps = list(CSRC.glob("*")) + [HERE.parent / "include" / "lambda_gpu.h"]
    newest = max(p.stat().st_mtime for p in deps)
    if lib_path.exists() and not force and lib_path.stat().st_mtime >= newest:
        return lib_path

    def compile_one(spec):
        src, defs, name = spec
        obj = out / (name + ".o")
        cmd = [nvcc(), *_flags(), *defs, *["-D" + d for d in defines], "-c", str(CSRC / src), "-o", str(obj)]
        if verbose and src.endswith(".cu"):
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed on %s:\n%s\n%s" % (src, r.stdout, r.stderr))
        return obj, r.stderr

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(compile_one, SOURCES))
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
