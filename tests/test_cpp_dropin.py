"""The C++ drop-in (spand_public_gb300/csrc/tree.h) as the reference's own driver uses it.

tests/cpp/cli_flow.cpp follows the reference command-line driver (tests/spaND.cpp:208-367):
setters, partition, assemble, factorize inside try/catch, print_log, get_stop / nnz, a
solve and CG.  It is compiled with g++ against tree.h and linked with the product library;
the CPU test only builds it, the GPU test runs it and compares what it prints with the
same problem through the C ABI.
"""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "cli_flow.cpp")
CSRC = os.path.join(ROOT, "spand_public_gb300", "csrc")
OUT = os.path.join(ROOT, "spand_public_gb300", "_build", "cli_flow")


def _cuda_home():
    from spand_public_gb300 import build

    return build._cuda_home()


def _compile():
    from spand_public_gb300 import build

    lib = build.build()
    cuda = _cuda_home()
    libdir = os.path.dirname(lib)
    cudalib = [d for d in (os.path.join(cuda, "lib64"), os.path.join(cuda, "lib")) if os.path.isdir(d)]
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    cmd = ["g++", "-std=c++17", "-O1", "-I", CSRC, "-I", os.path.join(cuda, "include"), SRC, "-o", OUT,
           "-L", libdir, "-lspand_gb300", f"-Wl,-rpath,{libdir}"]
    for d in cudalib:
        cmd += ["-L", d, f"-Wl,-rpath,{d}"]
    cmd += ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return OUT


def test_cli_flow_compiles_against_tree_h():
    assert os.path.exists(_compile())


def _values(out):
    return dict(re.findall(r"^<<<<(\w+)=(\S+)$", out, re.M))


@pytest.mark.gpu
@pytest.mark.parametrize("n,dim,levels,tol,fp32", [(32, 2, 5, 1e-2, 0), (16, 3, 6, 1e-2, 0), (16, 3, 6, 1e-2, 1)])
def test_cli_flow_runs(n, dim, levels, tol, fp32):
    import spand_public_gb300 as pkg
    from spand_public_gb300 import problems as P

    exe = _compile()
    r = subprocess.run([exe, str(n), str(dim), str(levels), str(tol), str(fp32)], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    v = _values(r.stdout)
    assert "<<<<OK" in r.stdout and v["nonspd_throws"] == "1"
    assert "lvl |" in r.stdout  # print_log's table
    # the same problem through the C ABI: identical ordering-dependent quantities
    A = P.neglapl(n, dim)
    t = pkg.Tree(levels)
    t.set_verb(False)
    t.set_use_geo(True)
    t.set_Xcoo(P.linspace_nd(n, dim))
    t.set_tol(tol)
    t.set_fp32(bool(fp32))
    t.partition(A)
    t.assemble(A)
    t.factorize()
    assert int(v["N"]) == A.shape[0]
    assert int(v["stop"]) == t.get_stop()
    assert int(v["nnzfact"]) == t.nnz()
    assert 1 <= int(v["CG"]) <= 30
