"""Writes srgb_tables.h: the sRGB transfer-function tables of the extension profile.

Both the CUDA kernels and the CPU oracle include the generated header, so decode and encode give
the same binary32 values on every machine without evaluating pow() at run time.

  kSrgbToLinear[k]      = EOTF(k / 255) for k = 0..255 (IEC 61966-2-1: c <= 0.04045 ? c / 12.92
                          : ((c + 0.055) / 1.055) ** 2.4), rounded to binary32.
  kSrgbEncodeThreshold[k] = EOTF((k - 0.5) / 255) for k = 1..255 ([0] = 0 is unused): a linear value
                          v encodes to the unorm8 k = #{k in 1..255 : v >= threshold[k]}, i.e. the
                          sRGB-encoded value rounded to the nearest unorm8 (ties up); NaN and
                          negative values give 0.

Run: python gen_srgb_tables.py  (rewrites srgb_tables.h beside this script).
"""

import os
import struct


def eotf(c: float) -> float:
    return c / 12.92 if c <= 0.04045 else ((c + 0.055) / 1.055) ** 2.4


def f32(x: float) -> float:
    return struct.unpack("<f", struct.pack("<f", x))[0]


def literal(x: float) -> str:
    return "0.0f" if x == 0.0 else f32(x).hex() + "f"


def table(name: str, values) -> str:
    rows = []
    for i in range(0, 256, 4):
        rows.append("    " + ", ".join(literal(v) for v in values[i:i + 4]) + ",")
    return f"GBR_TABLE_QUAL float {name}[256] = {{\n" + "\n".join(rows) + "\n};\n"


def main() -> None:
    decode = [eotf(k / 255.0) for k in range(256)]
    thresholds = [0.0] + [eotf((k - 0.5) / 255.0) for k in range(1, 256)]
    assert all(f32(a) < f32(b) for a, b in zip(thresholds[1:], thresholds[2:]))
    out = [
        "// srgb_tables.h — generated by gen_srgb_tables.py; do not edit.",
        "// sRGB decode (unorm8 -> linear) and encode thresholds (linear -> unorm8) of the extension",
        "// profile, shared by the CUDA kernels and the CPU oracle.  The includer may define",
        "// GBR_TABLE_QUAL (e.g. `static __device__ const` for device code).",
        "#pragma once",
        "#ifndef GBR_TABLE_QUAL",
        "#define GBR_TABLE_QUAL static const",
        "#endif",
        "",
        "// EOTF(k / 255), k = 0..255",
        table("kSrgbToLinear", decode),
        "// EOTF((k - 0.5) / 255), k = 1..255; entry 0 unused",
        table("kSrgbEncodeThreshold", thresholds),
    ]
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "srgb_tables.h")
    with open(path, "w") as f:
        f.write("\n".join(out))


if __name__ == "__main__":
    main()
