"""Regenerate spectral_tables.h: the CIE 1931 2-degree colour-matching tables (360-830 nm, 1 nm)
and the Smits/Berge RGB-to-spectrum basis curves (32 samples over 380-720 nm).

These are published colourimetry data sets.  They are read from the reference's
src/core/SPD_Data.cpp so that the GPU module, the CPU oracle and the reference use bit-identical
constants.  Run by hand when the reference tree is available:

    python lambda_gb300/csrc/gen_spectral_tables.py <reference_root>/src/core/SPD_Data.cpp
"""
import re
import sys
import pathlib

NAMES = ["CIE_lambda", "CIE_X", "CIE_Y", "CIE_Z", "RGB2SpectLambda",
         "RGBRefl2SpectWhite", "RGBRefl2SpectCyan", "RGBRefl2SpectMagenta", "RGBRefl2SpectYellow",
         "RGBRefl2SpectRed", "RGBRefl2SpectGreen", "RGBRefl2SpectBlue",
         "RGBIllum2SpectWhite", "RGBIllum2SpectCyan", "RGBIllum2SpectMagenta", "RGBIllum2SpectYellow",
         "RGBIllum2SpectRed", "RGBIllum2SpectGreen", "RGBIllum2SpectBlue"]
OUT = {"CIE_lambda": "lgpu_cie_lambda", "CIE_X": "lgpu_cie_x", "CIE_Y": "lgpu_cie_y", "CIE_Z": "lgpu_cie_z",
       "RGB2SpectLambda": "lgpu_smits_lambda"}


def main(src):
    text = pathlib.Path(src).read_text(errors="replace")
    out = ["/* Generated by gen_spectral_tables.py: CIE 1931 2-degree observer (360-830 nm, 1 nm steps)",
           " * and Smits/Berge RGB->spectrum basis curves (32 samples, 380-720 nm).  Published data. */",
           "#pragma once", "#define LGPU_N_CIE 471", "#define LGPU_CIE_Y_INTEGRAL 106.856895f",
           "#define LGPU_N_SMITS 32", ""]
    basis = []
    for name in NAMES:
        m = re.search(r"const Real " + name + r"\[[^\]]*\]\s*=\s*\{([^}]*)\}", text)
        vals = [v.strip() for v in m.group(1).replace("\n", " ").split(",") if v.strip()]
        vals = [float(v.rstrip("fF")) for v in vals]
        if name in OUT:
            cname = OUT[name]
            out.append("#define %s_DATA \\" % cname.upper())
            for i in range(0, len(vals), 8):
                out.append("    " + ", ".join(repr(v) + "f" for v in vals[i:i + 8]) + ", \\")
            out.append("")
        else:
            basis.append((name, vals))
    # 14 basis curves in a fixed order: refl W C M Y R G B, illum W C M Y R G B
    out.append("#define LGPU_SMITS_BASIS_DATA \\")
    for name, vals in basis:
        assert len(vals) == 32, name
        out.append("    { /* %s */ \\" % name)
        for i in range(0, 32, 8):
            out.append("      " + ", ".join(repr(v) + "f" for v in vals[i:i + 8]) + ", \\")
        out.append("    }, \\")
    out.append("")
    out.append("#ifndef LGPU_TABLES_NO_HOST_ARRAYS")
    for cname in OUT.values():
        out.append("static const float %s[] = { %s_DATA };" % (cname, cname.upper()))
    out.append("static const float lgpu_smits_basis[14][32] = { LGPU_SMITS_BASIS_DATA };")
    out.append("#endif")
    dst = pathlib.Path(__file__).with_name("spectral_tables.h")
    dst.write_text("\n".join(out) + "\n")
    print("wrote", dst)


if __name__ == "__main__":
    if len(sys.argv) < 2:
        raise SystemExit("usage: gen_spectral_tables.py <path of the reference's src/core/SPD_Data.cpp>")
    main(sys.argv[1])
