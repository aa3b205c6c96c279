"""The C++ shim of INTEGRATION.md, the binding a dCNS maintainer compiles in place of
impl/findSimilarFragmentsForPairedSequence4.cpp, defines exactly the two overloads the reference declares
(impl/findSimilarFragmentsForPairedSequence.h:26-42): compiled against the reference's own headers it links with a
caller of both declared overloads.  A mismatched signature would be a new overload, leaving the declared one
undefined at link time.  The C ABI is stubbed, so no GPU is needed; the test runs where the reference checkout is."""
import os
import re
import subprocess

import pytest

from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CALLER = r"""
#include "impl/findSimilarFragmentsForPairedSequence.h"
int main() {
  int8_t s[4] = {0, 1, 3, 4};
  int32_t n = 4, win = 38;
  std::string a, b;
  Scorei m(2, -3);
  std::vector<PairedSimilarFragment> f1 = findSimilarFragmentsForPairedSequence(
      s, s, s, s, n, n, win, 40, 0, -4, -2, 2, -3, m, 8, a, b, 0.1, 0.382291, 0.006662, 10, 20);
  std::vector<PairedSimilarFragment> f2 = findSimilarFragmentsForPairedSequence(
      s, s, s, s, n, n, win, 40, 0, -4, -2, -45, 0, 2, -3, m, 8, a, b, 0.1, 0.382291, 0.006662, 50, 20000, 10, 20);
  return (int)(f1.size() + f2.size());
}
"""

STUB = r"""
#include "dcns_gb300.h"
int dcns_ctx_create(int, size_t, dcns_ctx **out) { *out = 0; return DCNS_ERR_DEVICE; }
const char *dcns_last_error(const dcns_ctx *) { return "stub"; }
void dcns_params_default(dcns_params *) {}
int dcns_align_pairs(dcns_ctx *, const dcns_pair *, int64_t, const dcns_params *, int, dcns_results **) {
  return DCNS_ERR_DEVICE;
}
void dcns_results_free(dcns_results *) {}
"""


def _shim():
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    m = re.search(r"```cpp\n(// dcns_gb300_shim\.cpp.*?)```", text, re.S)
    assert m, "INTEGRATION.md holds no shim block"
    return m.group(1)


def test_shim_defines_the_reference_overloads(tmp_path):
    ref = O.REFERENCE_DIR
    if not os.path.isfile(os.path.join(ref, "impl", "findSimilarFragmentsForPairedSequence.h")):
        pytest.skip("reference checkout not present on this host")
    files = {"shim.cpp": _shim(), "caller.cpp": CALLER, "stub.cpp": STUB}
    for name, text in files.items():
        (tmp_path / name).write_text(text)
    flags = ["g++", "-std=gnu++14", "-include", "cstdint", "-w", "-I", ref, "-I", os.path.join(ROOT, "include")]
    objs = []
    for src in ["shim.cpp", "caller.cpp", "stub.cpp", os.path.join(ref, "model", "Score.cpp"),
                os.path.join(ref, "model", "PairedSimilarFragment.cpp")]:
        obj = str(tmp_path / (os.path.basename(src) + ".o"))
        path = src if os.path.isabs(src) else str(tmp_path / src)
        r = subprocess.run(flags + ["-c", path, "-o", obj], capture_output=True, text=True)
        assert r.returncode == 0, f"{src} does not compile:\n{r.stderr[-3000:]}"
        objs.append(obj)
    r = subprocess.run(["g++", "-o", str(tmp_path / "caller")] + objs, capture_output=True, text=True)
    assert r.returncode == 0, f"the shim does not define the declared overloads:\n{r.stderr[-3000:]}"
