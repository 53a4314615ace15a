"""Build oracle/_ref/libref_kat.so: the golden-vector driver (oracle/ref_kat.cpp) linked with nine of
the reference renderer's translation units, compiled with g++ from the reference tree where it lies.
TEST INFRASTRUCTURE ONLY; the output stays in oracle/_ref/ and never ships.

Only units that compile unmodified are used.  Embree is replaced by a declaration-only header
(oracle/ref_shim/embree3/rtcore.h); the units used never call it.  Every unit that includes the
shader graph (src/shading/graph/ShaderGraph.h) is unbuildable with g++: the header declares explicit
template specialisations at class scope.

    python oracle/build_ref.py [reference_root]      (default: /root/reference)
"""
import pathlib
import subprocess
import sys

HERE = pathlib.Path(__file__).resolve().parent
OUT = HERE / "_ref"
LIB = OUT / "libref_kat.so"
UNITS = ["shading/Fresnel.cpp", "shading/media/HenyeyGreenstein.cpp", "shading/media/HomogeneousMedium.cpp",
         "core/Spectrum.cpp", "core/SPD_Data.cpp", "sampling/Piecewise.cpp", "camera/Camera.cpp", "camera/Aperture.cpp",
         "image/TextureEncoding.cpp"]
# camera/Aperture.cpp instantiates the reference's texture class, whose Morton-order addressing calls the
# x86 BMI2 intrinsic _pdep_u64 (image/Texture.h:46): that unit needs -mbmi2 (this x86 build only).
UNIT_FLAGS = {"camera/Aperture.cpp": ["-mbmi2"]}


def _has_bmi2():
    try:
        return "bmi2" in pathlib.Path("/proc/cpuinfo").read_text().split()
    except OSError:
        return False


def build(ref_root="/root/reference", force=False):
    """Returns the library path, or None where it cannot be built here (no reference tree, or a
    host without the BMI2 instructions the reference's texture class needs)."""
    src = pathlib.Path(ref_root) / "src"
    if not src.is_dir() or not _has_bmi2():
        return None
    if LIB.exists() and not force and LIB.stat().st_mtime >= (HERE / "ref_kat.cpp").stat().st_mtime:
        return LIB
    OUT.mkdir(exist_ok=True)
    flags = ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-fvisibility=hidden", "-include", "cstring",
             "-I", str(src), "-I", str(src.parent), "-I", str(HERE / "ref_shim"), "-w"]
    objs = []
    for u in UNITS:
        obj = OUT / (u.replace("/", "_") + ".o")
        subprocess.run(flags + UNIT_FLAGS.get(u, []) + ["-c", str(src / u), "-o", str(obj)], check=True)
        objs.append(str(obj))
    drv = OUT / "ref_kat.o"
    subprocess.run(flags + ["-mbmi2", "-c", str(HERE / "ref_kat.cpp"), "-o", str(drv)], check=True)   # drives texture_t too
    subprocess.run(["g++", "-shared", "-o", str(LIB), str(drv), *objs, "-Wl,--no-undefined"], check=True)
    return LIB


if __name__ == "__main__":
    print(build(*(sys.argv[1:2] or ["/root/reference"]), force=True))
