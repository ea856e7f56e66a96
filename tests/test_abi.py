"""The C-ABI library builds, loads and exports every symbol include/*.h declares."""
import ctypes
import glob
import os
import re

import flock_challenge_gb300 as F

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(flock_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return names


def test_library_exports_declared_symbols():
    F.lib()
    lib = ctypes.CDLL(F.lib_path())
    names = declared_symbols()
    assert "flock_witness" in names and "flock_commit" in names
    for n in sorted(names):
        assert hasattr(lib, n), f"missing export {n}"


def test_version_string():
    assert b"sm_103a" in F.lib().flock_version()


def test_create_without_gpu_reports_error():
    import torch
    if torch.cuda.is_available():
        return
    h = ctypes.c_void_p()
    assert F.lib().flock_create(0, 0, ctypes.byref(h)) != 0


def test_footprint_estimate_is_monotone():
    fp = [F.footprint_bytes(l) for l in range(8, 22)]
    assert all(b > a for a, b in zip(fp, fp[1:]))
    assert 7 << 30 < F.footprint_bytes(18) < 9 << 30
