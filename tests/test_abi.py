"""The C-ABI libraries load and export every entry point include/*.h declares
(no compute calls: these run without a GPU)."""
import ctypes
import os
import re

from conftest import REPO
from nrltb import abi, build


def _declared(header):
    txt = open(os.path.join(REPO, "include", header)).read()
    return set(re.findall(r"^\s*(?:int|void|long long|const char \*)\s*\**\s*(nrltb_\w+)\s*\(", txt, re.M))


def test_library_builds_and_exports_all_symbols():
    build.build_all()
    lib = ctypes.CDLL(abi.GPU_LIB)
    names = _declared("nrltb.h") | _declared("nrltb_input.h") | _declared("nrltb_bench.h")
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_abi_version_and_error_string():
    lib = abi.load_gpu()
    assert lib.nrltb_abi_version() == 2
    assert isinstance(lib.nrltb_last_error(), bytes)


def test_host_library_symbols():
    lib = ctypes.CDLL(abi.HOST_LIB)
    for n in _declared("nrltb_input.h"):
        assert hasattr(lib, n), n


def test_bad_arguments_fail_cleanly():
    lib = abi.load_gpu()
    # null context / pointers are rejected before any device work
    assert lib.nrltb_bande(None, None, None, None, None, None) == abi.NRLTB_E_ARG
    assert lib.nrltb_fetch(None, None) == abi.NRLTB_E_ARG
    assert lib.nrltb_ctx_create(None, 0) == abi.NRLTB_E_ARG
    assert lib.nrltb_nparams(2) == 330 and lib.nrltb_nparams(1) == 97


def test_struct_layouts_match_the_header(tmp_path):
    """Every field offset and struct size of include/nrltb.h, as the C compiler
    lays them out, equals the ctypes mirror the tests and the benchmark use."""
    import subprocess
    structs = {"nrltb_structure": abi.Structure_, "nrltb_params": abi.Params_, "nrltb_kmesh": abi.KMesh_,
               "nrltb_opts": abi.Opts_, "nrltb_pairs": abi.Pairs_, "nrltb_result": abi.Result_}
    src = ["#include <stdio.h>", "#include <stddef.h>", '#include "nrltb.h"', "int main(void) {"]
    for cname, py in structs.items():
        src.append('printf("%s size %%zu\\n", sizeof(%s));' % (cname, cname))
        for fname, _ in py._fields_:
            src.append('printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, fname, cname, fname))
    src.append("return 0; }")
    c = tmp_path / "layout.c"
    c.write_text("\n".join(src) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=gnu11", "-I", os.path.join(REPO, "include"), str(c), "-o", str(exe)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        a, b, v = line.split()
        got[(a, b)] = int(v)
    for cname, py in structs.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)
