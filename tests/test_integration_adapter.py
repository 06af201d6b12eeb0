"""The bound plugin that INTEGRATION.md tells a maintainer to add
(`bound_flowshop_gb300`, its first C++ block) compiles against the
reference's own plugin base (headers/bound_abstract.h) and this library's
C-ABI header, and is usable through a bound_abstract pointer — so the
documented binding matches the interface it claims to drop into.

Runs where the reference tree is present (the build container); elsewhere
it is skipped. The headers the reference leaves out come from the oracle's
shims (oracle/ref_shim), as for the oracle's own reference build."""
import os
import re
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def reference_dir():
    """WSBB_REFERENCE_DIR, else the tree oracle/build.sh compiled the
    reference from (recorded in oracle/_ref/reference_dir); None if neither."""
    ref = os.environ.get("WSBB_REFERENCE_DIR")
    if not ref:
        rec = os.path.join(ROOT, "oracle", "_ref", "reference_dir")
        if os.path.exists(rec):
            with open(rec) as f:
                ref = f.read().strip()
    return ref if ref and os.path.isdir(os.path.join(ref, "headers")) else None


def test_documented_bound_plugin_compiles_against_the_reference_interface():
    REF = reference_dir()
    if REF is None or shutil.which("g++") is None:
        pytest.skip("reference tree not given (WSBB_REFERENCE_DIR) nor built by "
                    "oracle/build.sh, or g++ not available")
    with open(os.path.join(ROOT, "INTEGRATION.md")) as f:
        blocks = re.findall(r"```cpp\n(.*?)```", f.read(), flags=re.S)
    plugin = blocks[0]
    assert "struct bound_flowshop_gb300 : public bound_abstract" in plugin
    with tempfile.TemporaryDirectory() as d:
        with open(os.path.join(d, "bound_flowshop_gb300.h"), "w") as f:
            f.write(plugin)
        with open(os.path.join(d, "use.cpp"), "w") as f:
            f.write('#include "bound_flowshop_gb300.h"\n'
                    "int main() {\n"
                    "  bound_flowshop_gb300 b;\n"
                    "  bound_abstract *a = &b;  // the reference's plugin base\n"
                    "  int perm[4] = {0, 1, 2, 3}, couts[2];\n"
                    "  if (0) a->bornes_calculer(perm, -1, 4, couts, 99999);\n"
                    "  return 0;\n"
                    "}\n")
        shim = os.path.join(ROOT, "oracle", "ref_shim")
        cmd = ["g++", "-std=gnu++17", "-fsyntax-only", "-w",
               "-I", os.path.join(REF, "src"), "-I", os.path.join(shim, "src"),
               "-I", os.path.join(shim, "headers"), "-I", os.path.join(REF, "headers"),
               "-I", os.path.join(ROOT, "include"), os.path.join(d, "use.cpp")]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-2000:]
