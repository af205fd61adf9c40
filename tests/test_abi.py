"""The C-ABI library loads and exports every declared symbol (CPU only; no
compute calls), and host-only planning enforces LibreTT's input rules."""
import re
import subprocess
from pathlib import Path

import pytest

import librett_gb300 as L
from librett_gb300 import _lib

ROOT = Path(__file__).resolve().parents[1]


def _exported():
    out = subprocess.run(["nm", "-D", "--defined-only", str(_lib.LIB_PATH)], check=True,
                         capture_output=True, text=True).stdout
    return {line.split()[-1] for line in out.splitlines() if line.strip()}


def test_c_header_symbols_exported():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        names |= set(re.findall(r"^\s*(?:[\w\*]+\s+)+\**(librett_c_\w+)\s*\(", text, re.M))
    assert names, "no extern C declarations found"
    exported = _exported()
    missing = sorted(n for n in names if n not in exported)
    assert not missing, missing
    lib = _lib.load()
    for n in names:
        getattr(lib, n)
    assert names == {n for n, _, _ in _lib.C_FUNCTIONS}


def test_cxx_symbols_match_librett_mangling():
    exported = _exported()
    for sym in _lib.CXX_SYMBOLS:
        assert sym in exported, sym
    # the C++ declarations of include/librett.h: LibreTT's six plus grouped execution
    text = (ROOT / "include" / "librett.h").read_text()
    decls = set(re.findall(r"^(?:void|librettResult)\s+(librett\w+)\(", text, re.M))
    assert decls == {"librettInitialize", "librettFinalize", "librettPlan", "librettPlanMeasure",
                     "librettDestroy", "librettExecute", *_lib.CXX_GROUP_SYMBOLS}
    demangled = subprocess.run(["nm", "-DC", "--defined-only", str(_lib.LIB_PATH)],
                               capture_output=True, text=True, check=True).stdout
    for name in _lib.CXX_GROUP_SYMBOLS:
        assert re.search(rf"\b{name}\(", demangled), name


def test_result_codes_and_strings():
    lib = _lib.load()
    names = [lib.librett_c_result_string(i).decode() for i in range(6)]
    assert names == ["LIBRETT_SUCCESS", "LIBRETT_INVALID_PLAN", "LIBRETT_INVALID_PARAMETER",
                     "LIBRETT_INVALID_DEVICE", "LIBRETT_INTERNAL_ERROR", "LIBRETT_UNDEFINED_ERROR"]


@pytest.mark.parametrize("dims,perm,es", [
    ([4, 4], [0, 0], 4),        # not a permutation
    ([4, 4], [0, 2], 4),        # out of range
    ([4, 0], [1, 0], 4),        # zero dim
    ([4, -3], [1, 0], 8),       # negative dim
    ([4, 4], [1, 0], 2),        # element size
    ([4, 4], [1, 0], 12),
    ([2] * 17, list(range(17)), 4),  # rank above the engine limit
    ([1 << 21, 1 << 20], [1, 0], 4),  # more than 2^40 elements
])
def test_invalid_inputs_rejected(dims, perm, es):
    with pytest.raises(L.LibrettError) as e:
        L.describe(dims, perm, es)
    assert e.value.code == L.LIBRETT_INVALID_PARAMETER


def test_plan_and_execute_without_device_fail_cleanly():
    # Without a GPU the runtime reports no device: planning returns an error
    # code instead of crashing (no kernels are launched).
    import torch
    if torch.cuda.is_available():
        pytest.skip("device present")
    rc, _ = L.librettPlan([8, 8], [1, 0], 4, None)
    assert rc == L.LIBRETT_INTERNAL_ERROR
    assert L.librettExecute(123456, 0, 0) == L.LIBRETT_INVALID_PLAN
    assert L.librettDestroy(123456) == L.LIBRETT_INVALID_PLAN


def test_plan_batch_arguments():
    """librett_c_plan_batch refuses missing arrays before planning anything."""
    lib = _lib.load()
    assert lib.librett_c_plan_batch(0, None, None, None, None, None, 0, None, None) == 0
    assert lib.librett_c_plan_batch(-1, None, None, None, None, None, 0, None, None) == 2
    assert lib.librett_c_plan_batch(2, None, None, None, None, None, 0, None, None) == 2
