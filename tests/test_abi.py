"""The C ABI without a GPU: the library loads, exports every function the
headers declare, and the ctypes mirror has the C struct layout."""
import ctypes
import os
import re
import subprocess
import tempfile

import pytest

from conftest import ROOT

HEADERS = [os.path.join(ROOT, "include", h) for h in ("gbba.h", "gbtri.h", "gbsfm.h")]


def declared_functions():
    names = []
    for h in HEADERS:
        src = open(h).read()
        names += re.findall(r"^\s*(?:gbba_status|void|int|int64_t|const char\*)\s+(gb\w+)\s*\(", src, re.M)
    return sorted(set(names))


def test_headers_declare_what_the_mirror_lists(abi):
    assert declared_functions() == sorted(abi.EXPORTED_SYMBOLS)


def test_library_exports_every_declared_symbol(gb):
    lib = gb.lib()
    for name in declared_functions():
        assert hasattr(lib, name), name
    assert lib.gbba_abi_version() == 1
    assert lib.gbba_status_string(3) == b"out of device memory"


def test_no_device_is_reported_not_faked(gb, abi):
    from conftest import gpu_available
    if gpu_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    assert gb.lib().gbba_create(0, ctypes.byref(h)) == abi.ERROR_NO_DEVICE


def test_struct_layout_matches_c(abi):
    fields = {"gbba_problem": abi.GbbaProblem, "gbba_options": abi.GbbaOptions, "gbba_summary": abi.GbbaSummary,
              "gbba_tuning": abi.GbbaTuning, "gbsfm_camera": abi.GbsfmCamera,
              "gbsfm_residual_stats": abi.GbsfmResidualStats}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "gbba.h"', '#include "gbsfm.h"', "int main(void){"]
    for cname, cls in fields.items():
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for f, _ in cls._fields_:
            lines.append(f'printf("{cname}.{f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0;}")
    d = tempfile.mkdtemp()
    c = os.path.join(d, "layout.c")
    open(c, "w").write("\n".join(lines))
    exe = os.path.join(d, "layout")
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
    out = dict(l.rsplit(" ", 1) for l in subprocess.run([exe], capture_output=True, text=True).stdout.split("\n") if l)
    for cname, cls in fields.items():
        assert int(out[cname]) == ctypes.sizeof(cls), cname
        for f, _ in cls._fields_:
            assert int(out[f"{cname}.{f}"]) == getattr(cls, f).offset, f"{cname}.{f}"


def test_default_options_agree(gb, abi):
    o = abi.GbbaOptions()
    gb.lib().gbba_default_options(ctypes.byref(o))
    p = abi.default_options()
    for f, _ in abi.GbbaOptions._fields_:
        assert getattr(o, f) == getattr(p, f), f
