"""The C-ABI library builds for sm_103a, loads, and exports every entry point
declared in include/sg_solver.h (no device needed)."""
import os
import re
import subprocess

import pytest

import specfem3d_geotech_gb300 as sg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    with open(os.path.join(ROOT, "include", "sg_solver.h")) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sg_[a-z0-9_]+)\s*\(", text)))


def test_header_lists_the_package_exports():
    assert set(declared_symbols()) == set(sg.EXPORTED)


def test_library_exports_every_declared_symbol(built_lib):
    L = sg.lib()
    for name in declared_symbols():
        assert hasattr(L, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", built_lib], capture_output=True, text=True).stdout
    for name in declared_symbols():
        assert re.search(rf"\bT {name}\b", out), name


def test_build_targets_sm103a_only():
    from specfem3d_geotech_gb300 import build
    flags = " ".join(build.FLAGS)
    assert "arch=compute_103a,code=sm_103a" in flags
    assert flags.count("-gencode") == 1


def test_no_device_is_reported_not_faked(built_lib):
    """Without a GPU the context cannot be created; nothing falls back to the CPU."""
    import ctypes
    L = sg.lib()
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a device is present")
    h = L.sg_create(0, 0)
    assert not h
    assert L.sg_create_status() == sg.SG_ERR_NODEVICE
    with pytest.raises(sg.SgError):
        sg.Context(0)
    del ctypes


def declared_prototypes():
    """{name: number of parameters} of every function declared in the header."""
    with open(os.path.join(ROOT, "include", "sg_solver.h")) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    out = {}
    for m in re.finditer(r"\b(sg_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;", text, flags=re.S):
        args = m.group(2).strip()
        out[m.group(1)] = 0 if args in ("", "void") else args.count(",") + 1
    return out


def test_ctypes_signatures_match_the_header(built_lib):
    """Every entry point the Python mirror declares argtypes for takes the
    header's number of parameters (a miscount would pass garbage through the C ABI)."""
    L = sg.lib()
    protos = declared_prototypes()
    assert set(protos) == set(declared_symbols())
    checked = 0
    for name, nargs in protos.items():
        argtypes = getattr(getattr(L, name), "argtypes", None)
        if argtypes is None:
            continue
        assert len(argtypes) == nargs, (name, len(argtypes), nargs)
        checked += 1
    assert checked >= len(protos) - 3   # all but argument-less calls carry argtypes
