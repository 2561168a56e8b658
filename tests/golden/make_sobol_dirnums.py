"""Recover Sobol direction numbers (degree s, coefficients a, initial m_1..m_s)
from the reference's generator matrices and write them as C++ source.

The reference ships its 256-dimension, 32-bit Sobol generator matrices as a
table (src/math/SobolMatrices256x32.h).  The renderer needs exactly those
matrices, so this script finds, for every dimension, the primitive-polynomial
recurrence (Bratley & Fox; Joe & Kuo 2008)

    m_i = 2 a_1 m_{i-1} ^ 4 a_2 m_{i-2} ^ ... ^ 2^{s-1} a_{s-1} m_{i-s+1} ^ 2^s m_{i-s} ^ m_{i-s}

that reproduces the columns V_i = m_i << (32 - i), checks that regenerating
the matrices gives the table back bit for bit, and writes the compact
direction numbers to ``zillumgl_gb300/csrc/sobol_dirnums.inc``.  The library
regenerates the matrices from them (csrc/scene.cpp), and tests/test_tables.py
checks the result against the reference table's SHA-256.  Run once where the
reference sources are present ($ZGL_REFERENCE_TREE names the tree); the
output is committed.
"""
from __future__ import annotations

import os
import re
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
OUT = ROOT / "zillumgl_gb300" / "csrc" / "sobol_dirnums.inc"
SRC = Path(os.environ.get("ZGL_REFERENCE_TREE", "/root/reference")) / "src" / "math" / "SobolMatrices256x32.h"


def read_matrices(path: Path) -> list[list[int]]:
    text = path.read_text()
    body = text[text.index("{") + 1: text.rindex("}")]
    vals = [int(x, 16) for x in re.findall(r"0x[0-9a-fA-F]+", body)]
    assert len(vals) == 256 * 32, len(vals)
    return [vals[d * 32:(d + 1) * 32] for d in range(256)]


def regenerate(s: int, a: int, m_init: list[int]) -> list[int]:
    m = list(m_init)
    for i in range(s, 32):  # 0-based i -> m_{i+1}
        v = m[i - s] ^ (m[i - s] << s)
        for k in range(1, s):
            if (a >> (s - 1 - k)) & 1:
                v ^= m[i - k] << k
        m.append(v)
    return [(m[i] << (31 - i)) & 0xFFFFFFFF for i in range(32)]


def recover(cols: list[int]) -> tuple[int, int, list[int]]:
    m = [cols[i] >> (31 - i) for i in range(32)]
    for s in range(1, 24):
        for a in range(1 << (s - 1)):
            if regenerate(s, a, m[:s]) == cols:
                return s, a, m[:s]
    raise ValueError("no recurrence found")


def main() -> int:
    mats = read_matrices(SRC)
    assert mats[0] == [1 << (31 - i) for i in range(32)], "dimension 0 is the van der Corput sequence"
    rows = []
    for d in range(1, 256):
        s, a, mi = recover(mats[d])
        assert regenerate(s, a, mi) == mats[d]
        rows.append((s, a, mi))
    lines = [
        "// sobol_dirnums.inc — direction numbers of Sobol dimensions 1..255:",
        "// {degree s, coefficient bits a, m_1 .. m_s}.  Dimension 0 is the",
        "// van der Corput sequence.  Generated by tests/golden/make_sobol_dirnums.py;",
        "// the matrices they generate equal the renderer's 256x32 table bit for bit.",
    ]
    for s, a, mi in rows:
        lines.append("{%d, %d, {%s}}," % (s, a, ", ".join(str(x) for x in mi)))
    OUT.write_text("\n".join(lines) + "\n")
    print(f"wrote {OUT} ({len(rows)} dimensions, max degree {max(r[0] for r in rows)})")
    return 0


if __name__ == "__main__":
    sys.exit(main())
