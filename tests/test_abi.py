"""The C-ABI library loads and exports every entry point include/*.h
declares. No compute call is made (CPU only)."""
import glob
import os
import re

import hann_gb300 as hg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[\w\s\*]+?\b(hann_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return names


def test_every_declared_symbol_exported(built):
    L = hg.load_library()
    decl = declared_functions()
    assert len(decl) >= 20
    missing = [n for n in sorted(decl) if not hasattr(L, n)]
    assert not missing, missing
    assert set(hg.EXPORTED) <= decl
    assert set(hg.EXPORTED_DIAG) <= decl


def test_library_is_in_tree(built):
    assert os.path.dirname(hg.LIB_PATH) == os.path.join(ROOT, "hann_gb300")
    assert os.path.exists(hg.LIB_PATH)


def test_missing_library_fails_loudly(tmp_path):
    import pytest
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        hg.load_library(str(tmp_path / "absent.so"))
