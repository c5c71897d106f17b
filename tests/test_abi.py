"""The C ABI: the library loads, exports every entry point include/monte.h
declares, and its presets equal the reference constants (no GPU needed)."""
import ctypes as C
import os
import re
import subprocess

import pytest

from monte_gb300 import abi
from monte_gb300.lib import LIB_PATH, MonteError, load

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(REPO, "include", f) for f in os.listdir(os.path.join(REPO, "include"))
           if f.endswith(".h")]


def declared_functions():
    names = set()
    for h in HEADERS:
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"\b(monte_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return names


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(LIB_PATH):
        from monte_gb300.build import build
        build()
    return load()


def test_exports_every_declared_symbol(lib):
    decl = declared_functions()
    assert "monte_fdk" in decl and "monte_ctx_create" in decl
    out = subprocess.run(["nm", "-D", "--defined-only", LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if ln.strip()}
    missing = sorted(decl - exported)
    assert not missing, missing
    for name in decl:
        getattr(lib, name)  # resolvable through ctypes too


def test_abi_version(lib):
    assert lib.monte_abi_version() == 1


def _same(a, b):
    return bytes(a) == bytes(b)


def test_fdk_presets_match_reference_constants(lib):
    g = abi.FdkGeom()
    lib.monte_fdk_geom_reference65(C.byref(g))
    assert _same(g, abi.fdk_geom_reference65())
    assert (g.nu, g.nv, g.n_views, g.du, g.sod, g.sdd, g.wdist) == (65, 65, 360, 0.5, 160, 220, 60)
    assert (g.s_begin, g.s_end, g.mask_radius, g.scale) == (125, 130, 118, 2.7)
    lib.monte_fdk_geom_reference325(C.byref(g))
    assert _same(g, abi.fdk_geom_reference325())
    assert (g.nu, g.du, g.mask_radius, g.scale, g.scale2) == (325, 0.1, 0, 2.7, 5.0)


def test_null_context_is_rejected(lib):
    g = abi.fdk_geom_reference65()
    assert lib.monte_fdk(None, C.byref(g), None, None, None, None, 0, 0, 0) == abi.MONTE_EINVAL
    assert lib.monte_ctx_destroy(None) == abi.MONTE_OK
    assert lib.monte_ctx_create(None, 0) == abi.MONTE_EINVAL
    assert lib.monte_last_error(None)


def test_context_without_gpu_fails_loudly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from monte_gb300.lib import Context
    with pytest.raises(MonteError) as e:
        Context(0)
    assert e.value.code in (abi.MONTE_ECUDA, abi.MONTE_EINVAL)
