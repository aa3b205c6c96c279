"""The drop-in boundary at link level: the committed shim (dcns_gb300/shim/dcns_gb300_shim.cpp) replaces
impl/findSimilarFragmentsForPairedSequence4.cpp in the reference's own executable.  Every source file that the
reference's CMakeLists.txt lists for its dCNS target (its command-line program, drivers and test sources) is compiled
unmodified, except findSimilarFragmentsForPairedSequence4.cpp, whose place the shim takes, and the whole is linked
with the engine library (dcns_gb300/_lib/libdcnsgpu.so) into a dCNS executable: every call of the six functions of
impl/findSimilarFragmentsForPairedSequence.h in the reference (controlLayer4.cpp:212,355,525,701,1411,1584,1928,1967
and getCnsForMultipleSpecies.cpp) then resolves to the shim.  The linked program runs its usage text (no GPU here).

Only where the reference checkout exists (x86: its sources select AVX2 code); objects are cached under oracle/_ref."""
import os
import platform
import re
import subprocess
from concurrent.futures import ThreadPoolExecutor

import pytest

from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM = os.path.join(ROOT, "dcns_gb300", "shim", "dcns_gb300_shim.cpp")
REPLACED = "impl/findSimilarFragmentsForPairedSequence4.cpp"
CACHE = os.path.join(ROOT, "oracle", "_ref", "linkcheck")


def _target_sources(ref):
    text = open(os.path.join(ref, "CMakeLists.txt")).read()
    m = re.search(r"add_executable\(dCNS(.*?)\)", text, re.S)
    assert m, "CMakeLists.txt has no dCNS target"
    srcs = []
    for tok in m.group(1).split():
        if tok.endswith(".cpp") and tok not in srcs:
            srcs.append(tok)
    return srcs


def _compile(args):
    src, obj, flags = args
    if os.path.exists(obj) and os.path.getmtime(obj) >= os.path.getmtime(src):
        return None
    r = subprocess.run(flags + ["-c", src, "-o", obj + ".tmp"], capture_output=True, text=True)
    if r.returncode != 0:
        return f"{src}:\n{r.stderr[-3000:]}"
    os.replace(obj + ".tmp", obj)
    return None


def test_shim_links_into_the_reference_executable():
    ref = O.reference_dir()
    if not ref:
        pytest.skip("reference checkout not present on this host")
    if platform.machine() not in ("x86_64", "AMD64"):
        pytest.skip("the reference's sources select x86 AVX2 code")
    import dcns_gb300
    lib = dcns_gb300.build()
    srcs = _target_sources(ref)
    assert REPLACED in srcs and "main.cpp" in srcs and "controlLayer4.cpp" in srcs
    os.makedirs(CACHE, exist_ok=True)
    gt = os.path.join(ref, "googletest", "googletest")
    flags = ["g++", "-O0", "-std=gnu++14", "-include", "cstdint", "-mavx2", "-w", "-I", ref, "-I",
             os.path.join(gt, "include"), "-I", gt, "-I", os.path.join(ROOT, "include")]
    jobs = [(os.path.join(ref, s), os.path.join(CACHE, s.replace("/", "_") + ".o"), flags)
            for s in srcs if s != REPLACED]
    jobs.append((os.path.join(gt, "src", "gtest-all.cc"), os.path.join(CACHE, "gtest-all.o"), flags))
    jobs.append((SHIM, os.path.join(CACHE, "shim.o"), flags))
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        errors = [e for e in ex.map(_compile, jobs) if e]
    assert not errors, "does not compile:\n" + "\n".join(errors)
    exe = os.path.join(CACHE, "dCNS")
    r = subprocess.run(["g++", "-o", exe] + [o for _, o, _ in jobs] +
                       [lib, "-Wl,-rpath," + os.path.dirname(lib), "-lpthread"], capture_output=True, text=True)
    assert r.returncode == 0, f"dCNS does not link with the shim in place:\n{r.stderr[-4000:]}"
    nm = subprocess.run(["nm", "-C", exe], capture_output=True, text=True).stdout
    for name in ("findSimilarFragmentsForPairedSequence(", "findSimilarFragmentsForPairedSequence_wighted(",
                 "findSimilarFragmentsForPairedSequence_wighted_1gap("):
        assert any(name in line and " T " in line for line in nm.splitlines()), name
    assert sum(" T findSimilarFragmentsForPairedSequence(" in line for line in nm.splitlines()) == 4
    run = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert "cut1Gap" in run.stdout + run.stderr  # the reference's usage text
