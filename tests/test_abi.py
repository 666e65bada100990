"""The C-ABI library: it builds, loads and exports every entry point that
include/tf_gpu.h declares; argument validation needs no GPU."""
import os
import re
import ctypes as C
import subprocess

import numpy as np

from tissuefolding_paperversion_gb300 import api, build, mesh

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "tf_gpu.h")


def declared_symbols():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^TF_API\s+[\w\s\*]+?\b(tf_\w+)\s*\(", txt, flags=re.M)))


def test_header_declares_the_binding_list():
    assert declared_symbols() == sorted(api.EXPORTED)


def test_library_exports_every_declared_symbol():
    lib = build.build()
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing
    L = api.load()
    for s in declared_symbols():
        assert hasattr(L, s)


def test_bad_input_is_rejected_before_any_device_work():
    t = mesh.config_tiny(seed=1, n=3, n_layers=1)
    t.conn = t.conn.copy()
    t.conn[5] = t.n_nodes + 7
    try:
        api.Solver(t)
    except api.TfError as e:
        assert e.status == api.TF_BAD_INPUT
    else:
        raise AssertionError("out-of-range connectivity was accepted")


def test_bad_options_are_rejected_before_any_device_work():
    t = mesh.config_tiny(seed=1, n=3, n_layers=1)
    for kw in ({"precond": 4}, {"precond": -1}, {"krylov_method": 3}):
        try:
            api.Solver(t, **kw)
        except api.TfError as e:
            assert e.status == api.TF_BAD_INPUT, kw
        else:
            raise AssertionError(f"{kw} was accepted")


def test_status_strings():
    L = api.load()
    for code in range(9):
        assert L.tf_status_string(code)


def test_ctypes_structs_match_the_header_layout(tmp_path):
    """Every field of the structs the C ABI takes (tf_mesh, tf_material,
    tf_options, tf_step_stats) sits at the offset the header gives it, and the
    sizes agree: a probe compiled against include/tf_gpu.h prints them."""
    structs = [api.tf_mesh, api.tf_material, api.tf_options, api.tf_step_stats]
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "tf_gpu.h"', "int main(void) {"]
    for s in structs:
        n = s.__name__
        lines.append(f'  printf("{n} size %zu\\n", sizeof({n}));')
        for f, _ in s._fields_:
            lines.append(f'  printf("{n} {f} %zu\\n", offsetof({n}, {f}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "probe.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.dirname(HEADER), str(src), "-o", str(exe)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        *key, v = line.split()
        got[tuple(key)] = int(v)
    for s in structs:
        n = s.__name__
        assert got[(n, "size")] == C.sizeof(s), n
        for f, _ in s._fields_:
            assert got[(n, f)] == getattr(s, f).offset, (n, f)
