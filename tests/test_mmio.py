"""The MatrixMarket reader (include/mmio.h, csrc/mmio.cu) against the
oracle's restatement of the reference drivers' reading loop
(oracle/mmread.py: NIST banner and size line, then fscanf per entry,
test/dspmv_test_dgx1.cu:139-181; for large files also the same loop in C,
oracle_mm_read_fscanf).  Indices and values bit for bit."""
import ctypes as C

import numpy as np
import pytest

from oracle import mmread as R

BANNER = "%%MatrixMarket matrix coordinate {} {}\n"


def write(tmp_path, name, text):
    p = tmp_path / name
    p.write_bytes(text.encode("ascii"))
    return p


def check_same(path, expand=False, threads=0):
    from hpda_sblas_pnnl_gb300 import mmio
    code, m, n, r, c, v = R.read_coo(path, expand)
    mm, nn, rr, cc, vv = mmio.read_coo(path, expand_symmetric=expand, threads=threads)
    assert (mm, nn) == (m, n)
    np.testing.assert_array_equal(rr, r)
    np.testing.assert_array_equal(cc, c)
    assert vv.tobytes() == v.tobytes()       # bit for bit, signs of zeros included
    assert mmio.read_header(path)["typecode"] == code
    return rr, cc, vv


def test_real_general_with_comments_blank_lines_and_crlf(sblas_lib, tmp_path):
    text = (BANNER.format("Real", "General") + "% a comment\n%\n\n"
            "  4 5 7\r\n"
            "1 1 1.5e-300\r\n"
            "\t2 3 -0.0\n"
            "% a comment between entries\n"
            "3 5 1e308\n"
            "\n"
            "4 2 0.1\n"
            "4 4 123456789.123456789\n"
            "1 5 -2.2250738585072014e-308\n"
            "2 1 +7\n"
            "3 3 99\n")                     # beyond nnz: ignored, as the reference
    p = write(tmp_path, "a.mtx", text)
    r, c, v = check_same(p)
    assert r.tolist() == [0, 1, 2, 3, 3, 0, 1] and c.tolist() == [0, 2, 4, 1, 3, 4, 0]
    assert np.signbit(v[1]) and v[1] == 0.0


def test_integer_and_pattern_fields(sblas_lib, tmp_path):
    p = write(tmp_path, "i.mtx", BANNER.format("integer", "general") +
              "3 3 4\n1 1 5\n2 2 -3\n3 1 2147483647\n1 3 0\n")
    _, _, v = check_same(p)
    assert v.tolist() == [5.0, -3.0, 2147483647.0, 0.0]
    p = write(tmp_path, "p.mtx", BANNER.format("pattern", "general") +
              "3 4 3\n1 4\n3 2\n2 2\n")
    _, _, v = check_same(p)
    assert (v == 1.0).all()


@pytest.mark.parametrize("sym", ["symmetric", "skew-symmetric"])
def test_symmetric_files(sblas_lib, tmp_path, sym):
    p = write(tmp_path, "s.mtx", BANNER.format("real", sym) +
              "4 4 5\n1 1 2.0\n2 1 0.5\n3 3 1.0\n4 2 -1.25\n4 4 3.0\n")
    r, c, v = check_same(p)            # stored triangle only, as the reference
    assert r.size == 5
    r, c, v = check_same(p, expand=True)
    assert r.size == 7 and (r[5], c[5]) == (0, 1) and (r[6], c[6]) == (1, 3)
    sign = -1.0 if sym == "skew-symmetric" else 1.0
    assert v[5] == sign * 0.5 and v[6] == sign * -1.25


def test_empty_and_announced_zero(sblas_lib, tmp_path):
    from hpda_sblas_pnnl_gb300 import mmio
    p = write(tmp_path, "z.mtx", BANNER.format("real", "general") + "10 7 0\n")
    m, n, r, c, v = mmio.read_coo(p)
    assert (m, n, r.size) == (10, 7, 0)
    assert mmio.read_header(p) == {"m": 10, "n": 7, "nnz": 0, "typecode": "MCRG"}


@pytest.mark.parametrize("field,sym", [("real", "general"), ("pattern", "symmetric"),
                                       ("integer", "general")])
def test_large_file_threads_agree(sblas_lib, tmp_path, field, sym):
    """A 7 MB file, read with 1, 3 and all threads: identical results, equal
    to the oracle's."""
    rng = np.random.default_rng(7)
    nz = 250_000
    m, n = 90_000, 80_000
    r = rng.integers(1, m + 1, nz)
    c = rng.integers(1, n + 1, nz)
    lines = [BANNER.format(field, sym), "% generated\n", f"{m} {n} {nz}\n"]
    if field == "real":
        v = rng.standard_normal(nz) * 10.0 ** rng.integers(-30, 30, nz)
        lines += [f"{a} {b} {float(x)!r}\n" for a, b, x in zip(r, c, v)]
    elif field == "integer":
        v = rng.integers(-10**6, 10**6, nz)
        lines += [f"{a} {b} {x}\n" for a, b, x in zip(r, c, v)]
    else:
        lines += [f"{a} {b}\n" for a, b in zip(r, c)]
    p = write(tmp_path, "big.mtx", "".join(lines))
    base = check_same(p, expand=(sym != "general"), threads=1)
    for t in (3, 0):
        got = check_same(p, expand=(sym != "general"), threads=t)
        for x, y in zip(base, got):
            assert x.tobytes() == y.tobytes()
    # the reference's own loop restated in C (fscanf per entry; no expansion)
    from hpda_sblas_pnnl_gb300 import mmio
    from oracle import oracle as O
    fm, fn, fr, fc, fv = O.mm_read_fscanf(p)
    mm, nn, rr, cc, vv = mmio.read_coo(p, expand_symmetric=False)
    assert (fm, fn) == (mm, nn)
    assert fr.tobytes() == rr.tobytes() and fc.tobytes() == cc.tobytes()
    assert fv.tobytes() == vv.tobytes()


def test_scipy_written_file(sblas_lib, tmp_path):
    sp = pytest.importorskip("scipy.sparse")
    sio = pytest.importorskip("scipy.io")
    a = sp.random(500, 400, density=0.02, format="coo", random_state=3)
    p = tmp_path / "sc.mtx"
    sio.mmwrite(str(p), a, comment="written by scipy")
    r, c, v = check_same(p)
    d = np.zeros((500, 400))
    np.add.at(d, (r, c), v)
    np.testing.assert_array_equal(d, a.toarray())


@pytest.mark.parametrize("text,status,words", [
    ("not a banner\n1 1 1\n1 1 1.0\n", -8, "banner"),
    (BANNER.format("complex", "general") + "2 2 1\n1 1 1.0 2.0\n", -7, "complex"),
    ("%%MatrixMarket matrix array real general\n2 2\n1.0\n2.0\n3.0\n4.0\n", -7, "coordinate"),
    (BANNER.format("real", "general") + "3 3 4\n1 1 1.0\n2 2 2.0\n", -8, "premature"),
    (BANNER.format("real", "general") + "3 3 2\n1 1 1.0\n4 2 2.0\n", -8, "out of range"),
    (BANNER.format("real", "general") + "3 3 2\n1 1 1.0\n2 0 2.0\n", -8, "out of range"),
    (BANNER.format("real", "general") + "3 3 2\n1 1 abc\n2 2 2.0\n", -8, "value"),
    (BANNER.format("real", "general") + "3 3 2\n1 1\n2 2 2.0\n", -8, "value"),
    (BANNER.format("integer", "general") + "3 3 1\n1 1 2.5\n", -8, "value"),
    (BANNER.format("real", "general") + "3 x 2\n1 1 1.0\n", -8, "size"),
    (BANNER.format("real", "general") + "3 3 1\n- 1 1.0\n", -8, "row index"),
    (BANNER.format("real", "general") + "3 3 1\n1 2a 1.0\n", -8, "column index"),
    (BANNER.format("real", "general") + "3 3 1\n+-1 1 1.0\n", -8, "row index"),
    (BANNER.format("integer", "general") + "3 3 1\n1 1 1x\n", -8, "value"),
])
def test_malformed_files_fail_with_status(sblas_lib, tmp_path, text, status, words):
    from hpda_sblas_pnnl_gb300 import _lib, mmio
    p = write(tmp_path, "bad.mtx", text)
    with pytest.raises(_lib.SblasError) as e:
        mmio.read_coo(p)
    assert e.value.status == status and words in str(e.value), str(e.value)
    with pytest.raises(R.MMError):
        R.read_coo(p)


def test_real_values_of_every_digit_count(sblas_lib, tmp_path):
    """Values of 1 to 17 significant digits, decimal exponents -30 to 30,
    written in several forms (%g, %e, %f, leading '+', '.5', '5.', 'E'):
    the reader's exact short-number path (Clinger) and its strtod path give
    the same doubles as the Python and the C fscanf oracles, bit for bit."""
    rng = np.random.default_rng(23)
    vals = []
    for digits in range(1, 18):
        for ex in range(-30, 31, 3):
            x = float(rng.uniform(1, 10)) * 10.0 ** ex * (-1) ** int(rng.integers(2))
            vals += ["%.*g" % (digits, x), "%.*e" % (digits - 1, x), "%.*E" % (digits - 1, x)]
    vals += ["%.6f" % float(v) for v in rng.standard_normal(50)]
    vals += ["+1.5", ".5", "5.", "-.25e+3", "+0", "-0", "-0.0", "0e-400", "9007199254740992",
             "9007199254740993", "1e22", "1e23", "1e-22", "123456789012345e-22",
             "0.000000000000000000000000000001", "4.9406564584124654e-324", "inf", "-nan"]
    vals = [v for v in vals if v not in ("inf", "-nan")]    # the Python oracle refuses these
    lines = [BANNER.format("real", "general"), f"7 7 {len(vals)}\n"]
    lines += [f"{1 + i % 7} {1 + (i // 7) % 7} {v}\n" for i, v in enumerate(vals)]
    p = write(tmp_path, "digits.mtx", "".join(lines))
    rr, cc, vv = check_same(p, threads=1)
    check_same(p, threads=3)
    from oracle import oracle as O
    _, _, fr, fc, fv = O.mm_read_fscanf(p)
    assert fv.tobytes() == vv.tobytes()
    assert np.signbit(vv[vals.index("-0")]) and not np.signbit(vv[vals.index("+0")])


def test_integer_tokens_read_in_place(sblas_lib, tmp_path):
    """Indices and integer values as strtoll reads a whole token: signs,
    leading zeros (past 64 characters too), the long long extremes as
    values; a value beyond long long is refused."""
    text = (BANNER.format("integer", "general") + "5 5 5\n"
            "+1 1 -9223372036854775808\n"
            "0002 +003 9223372036854775807\n"
            + "0" * 70 + "4 5 -0\n"
            "5\t\t5\v+17\n"
            "1 5 000\n")
    p = write(tmp_path, "ints.mtx", text)
    rr, cc, vv = check_same(p)
    assert rr.tolist() == [0, 1, 3, 4, 0] and cc.tolist() == [0, 2, 4, 4, 4]
    assert vv.tolist() == [-2.0 ** 63, 2.0 ** 63, 0.0, 17.0, 0.0]
    from hpda_sblas_pnnl_gb300 import _lib, mmio
    p2 = write(tmp_path, "over.mtx", BANNER.format("integer", "general") +
               "2 2 1\n1 1 9223372036854775808\n")
    with pytest.raises(_lib.SblasError, match="value"):
        mmio.read_coo(p2)


def test_missing_file(sblas_lib, tmp_path):
    from hpda_sblas_pnnl_gb300 import _lib, mmio
    with pytest.raises(_lib.SblasError) as e:
        mmio.read_coo(tmp_path / "none.mtx")
    assert e.value.status == -1


def test_nist_entry_points(sblas_lib, tmp_path):
    """mm_read_banner / mm_read_mtx_crd_size on a FILE * as the reference's
    drivers call them, mm_typecode_to_str and mm_is_valid."""
    libc = C.CDLL(None)
    libc.fopen.restype = C.c_void_p
    libc.fopen.argtypes = [C.c_char_p, C.c_char_p]
    libc.fclose.argtypes = [C.c_void_p]
    libc.free.argtypes = [C.c_void_p]
    p = write(tmp_path, "n.mtx", "%%MatrixMarket MATRIX Coordinate Pattern Symmetric\n"
              "% c\n% c\n  12 12 30\n")
    f = libc.fopen(str(p).encode(), b"r")
    assert f
    code = C.create_string_buffer(4)
    m, n, nz = C.c_int(), C.c_int(), C.c_int()
    try:
        assert sblas_lib.mm_read_banner(f, code) == 0
        assert code.raw == b"MCPS"
        assert sblas_lib.mm_read_mtx_crd_size(f, C.byref(m), C.byref(n), C.byref(nz)) == 0
        assert (m.value, n.value, nz.value) == (12, 12, 30)
    finally:
        libc.fclose(f)
    s = sblas_lib.mm_typecode_to_str(b"MCPS")
    assert C.string_at(s) == b"matrix coordinate pattern symmetric"
    libc.free(s)
    assert sblas_lib.mm_typecode_to_str(b"XCPS") is None
    assert sblas_lib.mm_is_valid(b"MCRG") == 1
    assert sblas_lib.mm_is_valid(b"MCPK") == 0
    assert sblas_lib.mm_is_valid(b"MAPG") == 0
    assert sblas_lib.mm_is_valid(b"MCRH") == 0
    p = write(tmp_path, "nb.mtx", "%%MatrixMarket tensor coordinate real general\n1 1 0\n")
    f = libc.fopen(str(p).encode(), b"r")
    try:
        assert sblas_lib.mm_read_banner(f, code) == 15      # MM_UNSUPPORTED_TYPE
    finally:
        libc.fclose(f)


@pytest.mark.gpu
def test_file_to_csr_to_spmv(sblas_lib, cuda, tmp_path):
    """A file read, converted to CSR on the device and multiplied: equal to
    the oracle's read, coo2csr and CSR loop."""
    import torch
    from hpda_sblas_pnnl_gb300 import mmio, ops
    from oracle import oracle as O
    rng = np.random.default_rng(11)
    m, n, nz = 3_000, 2_500, 40_000
    r = rng.integers(1, m + 1, nz)
    c = rng.integers(1, n + 1, nz)
    v = rng.standard_normal(nz)
    p = write(tmp_path, "g.mtx", BANNER.format("real", "general") + f"{m} {n} {nz}\n" +
              "".join(f"{a} {b} {float(x)!r}\n" for a, b, x in zip(r, c, v)))
    mm, nn, rp, col, val = mmio.read_csr(p)
    _, _, _, orow, ocol, oval = R.read_coo(p)
    ov, op_, oc = O.coo2csr(m, n, oval, orow, ocol)
    np.testing.assert_array_equal(rp, op_)
    np.testing.assert_array_equal(col, oc)
    assert val.tobytes() == ov.tobytes()
    x = rng.standard_normal(n)
    y = torch.zeros(m, dtype=torch.float64, device=cuda)
    t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a)).to(device=cuda, dtype=dt)
    ops.csrmv(t(rp, torch.int32), t(col, torch.int32), t(val, torch.float64),
              t(x, torch.float64), y, 1.0, 0.0, n=n)
    ref = O.csr_spmv(m, n, op_, oc, ov, x, np.zeros(m))
    got = y.cpu().numpy()
    assert np.linalg.norm(got - ref) <= 1e-12 * np.linalg.norm(ref)
