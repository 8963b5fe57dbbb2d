"""The ctypes mirrors of the C ABI's structs (msplat_gb300/_native.py for
include/msplat_engine.h, msplat_gb300/api.py for the reference's
include/msplat_c_api.h) have the C layout: a small C program compiled against
the headers prints each struct's size and each field's offset, and they must
equal ctypes' (CPU only; needs gcc)."""
import ctypes as C
import os
import shutil
import subprocess

import pytest

from msplat_gb300 import _native as N
from msplat_gb300 import api as A

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# C name -> ctypes class
STRUCTS = {n: getattr(N, n) for n in ["MsplatGaussians", "MsplatAdamState", "MsplatStepArgs", "MsplatEngineStats",
                                       "MsplatMcmcStats", "MsplatGradients", "MsplatTuning"]}
STRUCTS.update({"MsplatConfig": A._MsplatConfig, "MsplatStats": A._Stats, "MsplatEvalMetrics": A._Eval,
                "MsplatPixelBuffer": A._Pixels})


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not available")
    lines = ["#include <stdbool.h>", "#include <stddef.h>", "#include <stdio.h>", '#include "msplat_engine.h"',
             '#include "msplat_c_api.h"', "int main(void) {"]
    for s, cls in STRUCTS.items():
        lines.append(f'    printf("{s} size %zu\\n", sizeof({s}));')
        for f in cls._fields_:
            lines.append(f'    printf("{s} {f[0]} %zu\\n", offsetof({s}, {f[0]}));')
    lines += ["    return 0;", "}"]
    d = tmp_path_factory.mktemp("layout")
    src, exe = d / "layout.c", d / "layout"
    src.write_text("\n".join(lines) + "\n")
    r = subprocess.run([gcc, "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr   # a ctypes field the header does not have fails here
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    res = {}
    for line in out.splitlines():
        s, k, v = line.split()
        res[(s, k)] = int(v)
    return res


@pytest.mark.parametrize("name", sorted(STRUCTS))
def test_ctypes_mirror_matches_header(c_layout, name):
    cls = STRUCTS[name]
    assert C.sizeof(cls) == c_layout[(name, "size")], name
    for f in cls._fields_:
        assert getattr(cls, f[0]).offset == c_layout[(name, f[0])], (name, f[0])
