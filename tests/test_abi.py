"""CPU-side checks of the drop-in boundary: the C ABI library loads, exports every
function include/pars_gb300.h declares, and the plan POD layout matches the
reference's scan_plan (no compute calls: this machine may have no GPU)."""
import ctypes
import os
import re

import pytest

from conftest import GRAMMARS, ROOT, plan_bytes

HEADER = os.path.join(ROOT, "include", "pars_gb300.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(pars_[a-z_0-9]+)\s*\(", src)))


@pytest.fixture(scope="module")
def L():
    from pars_gb300 import build
    build.build_all()
    from pars_gb300 import _lib
    return _lib.lib()


def test_header_declares_the_boundary():
    names = declared_functions()
    for must in ("pars_create", "pars_destroy", "pars_plan_load", "pars_scan_device",
                 "pars_scan_host", "pars_scan_chunk", "pars_reserve_struct"):
        assert must in names


def test_library_exports_every_declared_symbol(L):
    from pars_gb300 import _lib
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing
    # and the Python binding covers them all
    assert set(declared_functions()) <= set(_lib.SIGNATURES)


def test_plan_layout(L):
    assert L.pars_plan_bytes() == 3177
    assert L.pars_version() >= 1
    for g in GRAMMARS:
        assert len(plan_bytes(g)) == 3177


def test_null_arguments_are_rejected(L):
    assert L.pars_create(0, 0, None) == -22
    assert L.pars_destroy(None) == -22
    assert L.pars_plan_load(None, None, 0, None) == -22
