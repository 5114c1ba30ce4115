"""Pure-Python restatement of how the reference's drivers read a
MatrixMarket file, the checker of the library's reader (csrc/mmio.cu).

TEST INFRASTRUCTURE ONLY: imported by tests/, never by the product package.

The reference reads with the NIST "Matrix Market I/O library for ANSI C"
(its include/mmio.h declares mm_read_banner, mm_read_mtx_crd_size,
mm_typecode_to_str; mmio.c itself is not vendored and the header carries no
version) and the per-entry loop at test/dspmv_test_dgx1.cu:139-181 (the
same loop in dspmv_test_dgx2.cu and dspmv_test_smt.cu):

  * banner: five whitespace-separated tokens, the first starting with
    "%%MatrixMarket", the other four lower-cased: "matrix", coordinate |
    array, real | complex | pattern | integer, general | symmetric |
    hermitian | skew-symmetric (NIST mm_read_banner);
  * size line: the first line after the banner not starting with '%',
    holding "M N nz" (NIST mm_read_mtx_crd_size);
  * entries: nz lines "i j [v]" read with fscanf "%d %d %lg" (real),
    "%d %d %d" (integer, converted to double) or "%d %d" (pattern, value
    1.0); both indices minus one (dspmv_test_dgx1.cu:160-181).  Symmetric
    files are not expanded.

Python's float() rounds decimal strings correctly, as strtod (the converter
behind "%lg") does, so values compare bit for bit.  `expand` mirrors
off-diagonals after the stored entries, the library's optional extension.
"""
from __future__ import annotations

import numpy as np

TYPES = {
    1: {"coordinate": "C", "array": "A"},
    2: {"real": "R", "complex": "C", "pattern": "P", "integer": "I"},
    3: {"general": "G", "symmetric": "S", "hermitian": "H", "skew-symmetric": "K"},
}


class MMError(ValueError):
    pass


def read_banner(line: str) -> str:
    tk = line.split()
    if len(tk) < 5:
        raise MMError("premature end of file")
    if not tk[0].startswith("%%MatrixMarket"):
        raise MMError("no header")
    tk = [tk[0]] + [t.lower() for t in tk[1:5]]
    if tk[1] != "matrix":
        raise MMError("unsupported type")
    code = "M"
    for i in (1, 2, 3):
        if tk[i + 1] not in TYPES[i]:
            raise MMError("unsupported type")
        code += TYPES[i][tk[i + 1]]
    return code


def read_coo(path, expand: bool = False):
    """(typecode, m, n, row, col, val) of a coordinate file."""
    with open(path, "r", encoding="ascii", newline=None) as f:
        lines = f.read().split("\n")
    code = read_banner(lines[0])
    if code[1] != "C" or code[2] == "C":
        raise MMError("unsupported type")   # the reference's test programs read real, integer, pattern only
    k = 1
    while k < len(lines) and (not lines[k].strip() or lines[k].lstrip().startswith("%")):
        k += 1
    if k >= len(lines):
        raise MMError("premature end of file")
    try:
        m, n, nz = (int(t) for t in lines[k].split()[:3])
    except ValueError as e:
        raise MMError("bad size line") from e
    k += 1
    rows, cols, vals = [], [], []
    for line in lines[k:]:
        if len(rows) == nz:
            break
        tk = line.split()
        if not tk or tk[0].startswith("%"):
            continue
        try:
            i, j = int(tk[0]), int(tk[1])
            if not (1 <= i <= m and 1 <= j <= n):
                raise MMError("index out of range")
            if code[2] == "P":
                v = 1.0
            elif code[2] == "I":
                v = float(int(tk[2]))
            else:
                v = float(tk[2])
        except (ValueError, IndexError) as e:
            if isinstance(e, MMError):
                raise
            raise MMError("bad entry") from e
        rows.append(i - 1)
        cols.append(j - 1)
        vals.append(v)
    if len(rows) < nz:
        raise MMError("premature end of file")
    if expand and code[3] != "G":
        sign = -1.0 if code[3] == "K" else 1.0
        mr = [(c, r, sign * v) for r, c, v in zip(rows, cols, vals) if r != c]
        rows += [t[0] for t in mr]
        cols += [t[1] for t in mr]
        vals += [t[2] for t in mr]
    return (code, m, n, np.array(rows, dtype=np.int32), np.array(cols, dtype=np.int32),
            np.array(vals, dtype=np.float64))
