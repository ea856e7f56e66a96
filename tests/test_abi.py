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


def test_twiddle_classes_match_the_oracle_twiddles():
    """The narrow twiddle classes the multiply passes use (host arithmetic, no
    GPU) against the oracle's breadth-first twiddle table: byte k is the first
    layer from which every deeper layer's twiddles stay below 2^32, 2^40, 2^64
    and 2^72 (the OR of a layer's twiddles bounds them all)."""
    import numpy as np
    import oracle_lib as O

    L = F.lib()
    for dim in range(2, 23):
        tw = O.ntt_twiddles(dim).reshape(-1, 2)
        widths = []
        for layer in range(dim):
            seg = tw[(1 << layer) - 1:(1 << (layer + 1)) - 1]
            lo, hi = int(np.bitwise_or.reduce(seg[:, 0])), int(np.bitwise_or.reduce(seg[:, 1]))
            widths.append(64 + hi.bit_length() if hi else lo.bit_length())
        want = []
        for bound in (32, 40, 64, 72):
            first = dim
            for layer in range(dim - 1, -1, -1):
                if widths[layer] > bound:
                    break
                first = layer
            want.append(first)
        got = L.flock_ntt_twiddle_classes(dim)
        assert [(got >> (8 * k)) & 255 for k in range(4)] == want, (dim, widths)
    # the deepest layers of the 2^20-position L0 code: 20-, 37- and 69-bit twiddles
    got = L.flock_ntt_twiddle_classes(20)
    assert [(got >> (8 * k)) & 255 for k in range(4)] == [19, 18, 18, 17]
    assert L.flock_ntt_twiddle_classes(0) == -4 and L.flock_ntt_twiddle_classes(41) == -4
