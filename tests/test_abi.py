"""The C-ABI library loads and exports every entry point include/vclgb.h
declares (no GPU needed: nothing is called)."""
import os
import re
import subprocess

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "vclgb.h")
LIB = os.path.join(ROOT, "viennacl-dev_gb300", "libvclgb.so")


def declared():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"VCLGB_API\s+[\w\s\*]+?\b(vclgb\w+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(LIB):
        import __graft_entry__
        __graft_entry__.build()
    import vclgb
    return vclgb.load_library()


def test_every_declared_symbol_is_exported(lib):
    names = declared()
    assert len(names) >= 30
    for n in names:
        assert hasattr(lib, n), n


def test_only_the_abi_is_exported(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", LIB], capture_output=True, text=True,
                         check=True).stdout
    text_syms = [l.split()[-1] for l in out.splitlines() if " T " in l]
    assert text_syms and all(s.startswith("vclgb") for s in text_syms), text_syms
    assert sorted(text_syms) == declared()


def test_python_mirror_covers_the_abi(lib):
    import vclgb
    assert sorted(vclgb.SIGNATURES) == declared()
    assert lib.vclgbVersion().decode().startswith("vclgb")


def test_library_links_only_system_and_driver_libraries():
    out = subprocess.run(["ldd", LIB], capture_output=True, text=True).stdout
    assert "libtorch" not in out and "libc10" not in out
