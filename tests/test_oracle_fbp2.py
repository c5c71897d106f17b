"""The 2-D fan-beam FBP oracle (oracle/fbp2_oracle.c) against the reference
program recon/fbp2.cpp, compiled unmodified (tests/golden/fbp2.npz): the
filtered projections and the image must be equal bit for bit.  The preset
of the C ABI equals the reference's constants (no GPU needed)."""
import ctypes as C

import numpy as np

import oracle
from helpers import golden
from inputs import fdk_projections
from monte_gb300 import abi
from monte_gb300.lib import load


def test_fbp2_oracle_matches_reference_program():
    gold = golden("fbp2")
    g = abi.fbp2_geom_reference()
    proj = fdk_projections(360, 65, 1, int(gold["seed"])).reshape(360, 65)
    filt, img = oracle.fbp2(g, proj)
    assert np.array_equal(filt, gold["filtered"])
    assert np.array_equal(img, gold["image"])
    assert np.abs(img).max() > 0


def test_fbp2_preset_equals_reference_constants():
    lib = load()
    g = abi.Fbp2Geom()
    lib.monte_fbp2_geom_reference(C.byref(g))
    ref = abi.fbp2_geom_reference()
    for name, _ in abi.Fbp2Geom._fields_:
        assert getattr(g, name) == getattr(ref, name), name
