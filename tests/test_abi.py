"""The C-ABI library: it builds, loads and exports every entry point that
include/tf_gpu.h declares; argument validation needs no GPU."""
import os
import re
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
