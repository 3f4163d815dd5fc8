"""The C ABI library builds, loads and exports every function that
include/dsf_gb300.h declares (no GPU needed)."""
import ctypes
import os
import re
import subprocess

import pytest

from discamb_gb300 import build

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in os.listdir(os.path.join(REPO, "include")):
        if not h.endswith(".h"):
            continue
        text = open(os.path.join(REPO, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(dsf_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib_path():
    return build.build()


def test_header_declares_the_boundary():
    names = declared_functions()
    for required in ("dsf_engine_create", "dsf_structure_create_hc", "dsf_calculate", "dsf_calculate_atoms",
                     "dsf_calculate_device", "dsf_last_error"):
        assert required in names


def test_library_exports_every_declared_symbol(lib_path):
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\b(dsf_\w+)\b", out))
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing


def test_library_loads_and_reports_version(lib_path):
    lib = ctypes.CDLL(lib_path)
    assert lib.dsf_abi_version() == 1


def test_invalid_handles_are_rejected_without_a_device(lib_path):
    lib = ctypes.CDLL(lib_path)
    assert lib.dsf_engine_create(0, None) != 0
    assert lib.dsf_structure_destroy(None) != 0
    assert lib.dsf_calculate(None, 0, 0, None, None, None) != 0
    assert lib.dsf_calculate_atoms(None, 0, 0, None, None, None, None, None, None) != 0
