"""Phantom generators (CPU): the voxelised analytic phantom of
monte_cu/CBCT_real325.cu:916-928 and the label volume of
monte_cpp/make_image01.cpp."""
import numpy as np

from monte_gb300 import phantoms


def test_ca_rod_phantom_geometry():
    lab, vox, org, dens, mats = phantoms.ca_rod_labels(voxel_cm=0.2)
    assert lab.shape == (100, 100, 100) and org == (-10.0, -10.0, -10.0)
    assert dens == [0.0, 1.0, 1.55] and mats == [-1, 0, 1]
    v = vox ** 3
    # cylinder r = 10 cm, length 20 cm; eight rods r = 1.5 cm
    cyl = np.pi * 100.0 * 20.0
    rods = 8 * np.pi * 2.25 * 20.0
    assert abs((lab > 0).sum() * v / cyl - 1) < 0.01
    assert abs((lab == 2).sum() * v / rods - 1) < 0.02
    # rod centres 5 cm off the axis every 45 degrees in the y-z plane: the
    # x = 0 slice is symmetric under y -> -y, z -> -z and y <-> z
    sl = lab[:, :, 50]
    assert np.array_equal(sl, sl[::-1, ::-1])
    assert np.array_equal(sl, sl.T)
    # (y, z) = (5, 0) is Ca, the axis is water, a corner is air
    idx = lambda c: int((c + 10.0) / vox)
    assert lab[idx(0.0), idx(5.0), idx(0.0)] == 2
    assert lab[idx(0.0), idx(0.0), idx(0.0)] == 1
    assert lab[idx(9.5), idx(9.5), idx(0.0)] == 0


def test_sphere_phantom_matches_make_image01():
    lab = phantoms.sphere_labels_185()
    assert lab.shape == (325, 185, 185)
    assert lab[160, 90, 90] == 1 and lab[160, 90, 141] == 0 and lab[160, 90, 140] == 1
