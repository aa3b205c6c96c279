"""CPU-side checks of the C-ABI library: it builds for sm_103a, loads, exports every symbol include/dcns_gb300.h
declares, and refuses to run without a GPU (no CPU fallback).  No compute calls."""
import ctypes
import os
import re
import subprocess

import pytest

import dcns_gb300

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "dcns_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(dcns_[a-z_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def so_path():
    return dcns_gb300.build()


def test_library_exports_every_declared_symbol(so_path):
    syms = declared_symbols()
    assert len(syms) >= 15
    out = subprocess.run(["nm", "-D", "--defined-only", so_path], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r" T (dcns_\w+)", out))
    missing = [s for s in syms if s not in exported]
    assert not missing, missing
    lib = ctypes.CDLL(so_path)
    for s in syms:
        getattr(lib, s)


def test_params_default_matches_reference_globals(so_path):
    p = dcns_gb300.params()
    # controlLayer4.cpp:28-52 of the reference
    assert (p.match, p.mismatch, p.open1, p.ext1, p.open2, p.ext2) == (2, -3, -4, -2, -45, 0)
    assert (p.window, p.min_score, p.step, p.w, p.xdrop, p.zdrop, p.bandwidth) == (38, 40, 8, 10, 20, 50, 20000)
    assert (p.pvalue, p.lambda_, p.kvalue) == (0.1, 0.382291, 0.006662)


def test_no_gpu_fails_loudly(so_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(dcns_gb300.DcnsError):
        dcns_gb300.Engine(0)



def test_python_structs_match_the_c_layout(tmp_path):
    """The ctypes mirrors of the header's structs have the C compiler's size and field offsets (a mismatch would make
    the library write past the Python buffers)."""
    import shutil
    if not shutil.which("gcc"):
        pytest.skip("no C compiler")
    pairs = [("dcns_params", dcns_gb300.Params), ("dcns_pair", dcns_gb300.Pair), ("dcns_stats", dcns_gb300.Stats),
             ("dcns_serving_stats", dcns_gb300.ServingStats), ("dcns_tuning", dcns_gb300.Tuning),
             ("dcns_results", dcns_gb300.Results)]
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "dcns_gb300.h"', "int main(void) {"]
    for cname, py in pairs:
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:  # Python spells the C field `lambda` as lambda_
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname.rstrip("_")}));')
    lines.append("  return 0;\n}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        name, key, val = line.split()
        got[(name, key)] = int(val)
    for cname, py in pairs:
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)
