"""The drop-in headers from C and C++ callers (CPU only, no GPU calls).

C and C++ programs are compiled against include/spmv_kernel.h and
include/mmio.h, linked to libsblas_gb300.so and run through paths that need
no GPU (argument errors, host helpers, MatrixMarket banners).  Where the
reference's source tree is present, its unchanged test programs
(test/dspmv_test_{smt,dgx1,dgx2}.cu) are compiled and linked against this
library with the documented build command (nvcc, this repository's include
directory first, -lsblas_gb300 alone)."""
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from conftest import ROOT

INC = ROOT / "include"


def _reference_root() -> Path | None:
    """The reference's source tree: $SBLAS_REFERENCE_DIR, else the root that
    oracle/ref_build.sh compiled from (recorded in oracle/_ref/REFERENCE_DIR)."""
    env = os.environ.get("SBLAS_REFERENCE_DIR")
    if env:
        return Path(env)
    rec = ROOT / "oracle" / "_ref" / "REFERENCE_DIR"
    if rec.exists():
        return Path(rec.read_text().strip())
    return None


REFERENCE = _reference_root()

C_CALLER = r"""
#include <stdio.h>
#include "spmv_kernel.h"
#include "mmio.h"
int main(int argc, char **argv)
{
    int rowptr[4] = {0, 2, 2, 5}, col[5] = {0, 2, 1, 2, 0};
    double val[5] = {1, 2, 3, 4, 5}, x[3] = {1, 1, 1}, y[3] = {7, 8, 9};
    double alpha = 1.0, beta = 0.0;
    struct spmv_ret r = spMV_mgpu_baseline(3, 3, 5, &alpha, val, rowptr, col, x, &beta, y, 2);
    printf("%g %g %g %g %g\n", r.numa_part_time, r.part_time, r.comp_time, r.comm_time,
           r.merg_time);
    printf("%s|%d\n", sblas_last_error(), sblas_last_status());
    printf("%g %g %g\n", y[0], y[1], y[2]);
    printf("%d %d %d\n", get_row_from_index(3, rowptr, 0), get_row_from_index(3, rowptr, 2),
           get_row_from_index(3, rowptr, 4));
    FILE *f = fopen(argv[1], "r");
    MM_typecode t;
    int rc = mm_read_banner(f, &t);
    int M = 0, N = 0, nz = 0;
    int rc2 = mm_read_mtx_crd_size(f, &M, &N, &nz);
    fclose(f);
    printf("%d %d %c%c%c%c %d %d %d %d\n", rc, rc2, t[0], t[1], t[2], t[3], M, N, nz,
           mm_is_symmetric(t) ? 1 : 0);
    f = fopen(argv[2], "r");
    rc = mm_read_banner(f, &t);
    rc2 = mm_read_mtx_array_size(f, &M, &N);
    fclose(f);
    printf("%d %d %d %d %d\n", rc, rc2, mm_is_array(t) ? 1 : 0, M, N);
    double pv[5] = {0.1, -2.5e-7, 123456789.0, 3.0, -0.0};
    int iv[3] = {-1, 0, 2147483647};
    print_vec_double(pv, 5, "d");
    print_vec_int(iv, 3, "i");
    print_vec_int(iv, 0, "none");
    printf("%s\n", sblas_version());
    return 0;
}
"""

CXX_CALLER = r"""
#include "spmv_kernel.h"
#include <iostream>
int main(int argc, char **argv)
{
    spmv_ret a, b;
    a.init();
    b.init();
    b.comp_time = 3.0;
    b.merg_time = 1.0;
    a.add(b);
    a.add(b);
    a.avg(2);
    std::cout << a.to_string();
    int v[3] = {4, 5, 6};
    print_vec(v, 3, std::string("v"));
    checkCudaErrors(0);
    if (argc > 1) checkCudaErrors(35);
    std::cout << "after" << std::endl;
    return 0;
}
"""

MTX = "%%MatrixMarket matrix coordinate real symmetric\n% comment\n3 3 2\n1 1 1.0\n3 1 2.0\n"
MTX_ARRAY = "%%MatrixMarket matrix array real general\n%\n2 3\n1\n2\n3\n4\n5\n6\n"


def _tool(name):
    p = shutil.which(name)
    if p is None:
        pytest.skip(f"{name} not on PATH")
    return p


def _link_flags(lib_dir: Path) -> list[str]:
    return [f"-L{lib_dir}", "-lsblas_gb300", f"-Wl,-rpath,{lib_dir}"]


def test_c_caller_links_and_gets_statuses(sblas_lib, tmp_path):
    from hpda_sblas_pnnl_gb300 import _lib
    lib_dir = _lib.lib_path().parent
    src = tmp_path / "caller.c"
    src.write_text(C_CALLER)
    exe = tmp_path / "caller_c"
    subprocess.run([_tool("gcc"), "-std=c11", "-Wall", "-Werror", f"-I{INC}", str(src), "-o",
                    str(exe), *_link_flags(lib_dir)], check=True)
    mtx = tmp_path / "a.mtx"
    mtx.write_text(MTX)
    arr = tmp_path / "b.mtx"
    arr.write_text(MTX_ARRAY)
    out = subprocess.run([str(exe), str(mtx), str(arr)], check=True, capture_output=True,
                         text=True).stdout.splitlines()
    assert out[0] == "-1 -1 -1 -1 -1"                 # failure record, no exit
    msg, status = out[1].rsplit("|", 1)
    assert "ngpu" in msg and int(status) == -2        # SBLAS_ERR_NGPU
    assert out[2] == "7 8 9"                          # y untouched on failure
    rp = np.array([0, 2, 2, 5], dtype=np.int32)
    from hpda_sblas_pnnl_gb300 import api
    assert out[3] == " ".join(str(api.get_row_from_index(3, rp, i)) for i in (0, 2, 4))
    assert out[4] == "0 0 MCRS 3 3 2 1"
    assert out[5] == "0 0 1 2 3"
    # the reference's print_vec: "<s>: " then each value and a space (ostream
    # defaults, i.e. %g for doubles)
    assert out[6] == "d: " + "".join("%g " % v for v in (0.1, -2.5e-7, 123456789.0, 3.0, -0.0))
    assert out[7] == "i: -1 0 2147483647 "
    assert out[8] == "none: "
    assert out[9].startswith("sblas-gb300")


def test_cxx_caller_uses_member_functions_and_check_macro(sblas_lib, tmp_path):
    from hpda_sblas_pnnl_gb300 import _lib
    lib_dir = _lib.lib_path().parent
    src = tmp_path / "caller.cpp"
    src.write_text(CXX_CALLER)
    exe = tmp_path / "caller_cxx"
    subprocess.run([_tool("g++"), "-std=c++14", "-Wall", "-Werror", f"-I{INC}", str(src), "-o",
                    str(exe), *_link_flags(lib_dir)], check=True)
    ok = subprocess.run([str(exe)], check=True, capture_output=True, text=True)
    lines = ok.stdout.splitlines()
    assert lines[0] == "0,0,0,3,1"                    # numa_part, part, comm, comp, merg
    assert lines[1] == "v: 4 5 6 "
    assert lines[-1] == "after"
    bad = subprocess.run([str(exe), "fail"], capture_output=True, text=True)
    assert bad.returncode != 0 and "after" not in bad.stdout
    assert "CUDA error 35" in bad.stderr and "checkCudaErrors" not in bad.stderr


@pytest.mark.skipif(REFERENCE is None or not (REFERENCE / "test" / "dspmv_test_smt.cu").exists(),
                    reason="the reference's source tree is not present")
def test_reference_test_programs_relink_unchanged(sblas_lib, tmp_path):
    """The reference's own test programs, unchanged, compile against this
    repository's header (found before the reference's own include dir) and
    link to this library alone."""
    from hpda_sblas_pnnl_gb300 import _lib
    nvcc = _tool("nvcc")
    lib_dir = _lib.lib_path().parent
    procs = {}
    for name in ("smt", "dgx1", "dgx2"):
        src = REFERENCE / "test" / f"dspmv_test_{name}.cu"
        cmd = [nvcc, "-std=c++14", "-gencode", "arch=compute_103a,code=sm_103a",
               f"-I{INC}", f"-I{REFERENCE / 'include'}", str(src), "-o",
               str(tmp_path / f"test_{name}"), f"-L{lib_dir}", "-lsblas_gb300",
               "-Xlinker", f"-rpath={lib_dir}"]
        procs[name] = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                                       text=True)
    for name, p in procs.items():
        out, _ = p.communicate(timeout=600)
        assert p.returncode == 0, f"{name}:\n{out[-3000:]}"
        assert (tmp_path / f"test_{name}").exists()
