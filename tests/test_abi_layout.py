"""The ctypes mirrors of the C ABI's structs (unsupervised_growth_gb300/engine.py) have
the layout of include/ugrowth.h: the same size and the same offset for every field,
checked by compiling the header with the host C compiler.  No GPU is needed."""
import ctypes as C
import os
import shutil
import subprocess

import pytest

from unsupervised_growth_gb300 import engine as E

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PAIRS = [
    ("ug_synaptic_params", E.SynapticParams),
    ("ug_maturation_params", E.MaturationParams),
    ("ug_noise_params", E.NoiseParams),
    ("ug_connection_params", E.ConnectionParams),
    ("ug_network_desc", E.NetworkDesc),
    ("ug_network_info", E.NetworkInfo),
    ("ug_runtime_opts", E.RuntimeOpts),
    ("ug_group_item", E.GroupItem),
    ("ug_server_opts", E.ServerOpts),
    ("ug_request", E.Request),
    ("ug_request_info", E.RequestInfo),
    ("ug_topology_params", E.TopologyParams),
    ("ug_topology_info", E.TopologyInfo),
]


def c_layout(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "ugrowth.h"', "int main(void) {"]
    for cname, cls in PAIRS:
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for f, _ in cls._fields_:
            lines.append(f'printf("{cname}.{f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0; }")
    src, exe = tmp_path / "layout.c", tmp_path / "layout"
    src.write_text("\n".join(lines))
    subprocess.run([cc, "-std=c11", "-I" + os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return dict(line.rsplit(" ", 1) for line in out.splitlines())


def test_struct_layouts_match(tmp_path):
    got = c_layout(tmp_path)
    for cname, cls in PAIRS:
        assert int(got[cname]) == C.sizeof(cls), cname
        for f, _ in cls._fields_:
            assert int(got[f"{cname}.{f}"]) == getattr(cls, f).offset, f"{cname}.{f}"
