"""The C++ that INTEGRATION.md section 2 asks a maintainer to add to the
reference compiles: every ```cpp block of that section is placed in a member
function of a class derived from the reference's Simulation (so the
snippets' unqualified names -- Nodes, Elements, nNodes, dt, GrowthFunctions,
... -- resolve to the reference's own members) and checked with
``g++ -fsyntax-only`` against include/tf_gpu.h and the reference's headers
(GSL and Boost through the oracle's stand-in headers).  Runs where the
reference checkout is present."""
import os
import re
import shutil
import subprocess

import pytest

from oracle.oracle import REF_SRC

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _section_blocks():
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    sec = text[text.index("## 2."):text.index("## 3.")]
    return re.findall(r"```cpp\n(.*?)```", sec, flags=re.S)


def test_section_two_has_the_call_sequence():
    blocks = _section_blocks()
    assert len(blocks) >= 4
    joined = "\n".join(blocks)
    for call in ("tf_create", "tf_newton_step", "tf_get_positions", "tf_set_Fg", "tf_add_grid_growth",
                 "tf_set_packing"):
        assert call in joined, call


@pytest.mark.skipif(not os.path.isdir(REF_SRC) or shutil.which("g++") is None,
                    reason="the reference checkout (or g++) is not present")
def test_section_two_compiles_against_the_reference(tmp_path):
    blocks = _section_blocks()
    body = []
    for k, b in enumerate(blocks):
        includes = [ln for ln in b.splitlines() if ln.startswith("#include")]
        code = "\n".join(ln for ln in b.splitlines() if not ln.startswith("#include"))
        body.append((includes, f"    void snippet{k}() {{\n{code}\n    }}\n"))
    src = ['#include "Simulation.h"', '#include "GrowthFunctionTypes.h"', "#include <cmath>", "#include <cstdint>",
           "#include <vector>"]
    for inc, _ in body:
        src += inc
    src += ["struct GpuStepIntegration : Simulation {", "    tf_handle* gpuStep = nullptr;"]
    src += [code for _, code in body]
    src += ["};"]
    f = tmp_path / "integration_snippets.cpp"
    f.write_text("\n".join(src) + "\n")
    cmd = ["g++", "-std=gnu++14", "-include", "algorithm", "-fsyntax-only", "-w",
           "-I", os.path.join(ROOT, "oracle", "ref", "shim"), "-I", REF_SRC, "-I", os.path.join(ROOT, "include"),
           str(f)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
