"""The drop-in host programs read and write the reference's raw files."""
import os
import subprocess

import numpy as np
import pytest

from helpers import golden, past_end_voxels, rel_rms
from inputs import fdk_projections
from monte_gb300 import abi

pytestmark = pytest.mark.gpu
PROG = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "monte_gb300",
                    "programs")


def test_monte_fdk_program_matches_bp3d20(tmp_path):
    gold = golden("fdk65")
    proj = fdk_projections(360, 65, 65, int(gold["seed"]))
    proj.tofile(tmp_path / "mapg_0_20000h2oCa.raw")
    subprocess.run([os.path.join(PROG, "monte_fdk"), "--preset", "65"], cwd=tmp_path, check=True,
                   capture_output=True)
    xy = np.fromfile(tmp_path / "CBCTrecon\\xy2mh20kyu2.raw", np.float32).reshape(256, 256, 256)
    zy = np.fromfile(tmp_path / "CBCTrecon\\zy2mh20kyu2.raw", np.float32).reshape(256, 256, 256)
    filt = np.fromfile(tmp_path / "CBCTrecon\\map2mh20kyu2.raw", np.float32).reshape(360, 65, 65)
    keep = ~past_end_voxels(abi.fdk_geom_reference65())[:, :, 125:130]
    assert rel_rms(xy[:, :, 125:130][keep], gold["xy_slab"][keep]) < 1e-5
    assert np.array_equal(zy, xy.transpose(2, 1, 0))
    assert rel_rms(filt[gold["view_ids"]], gold["filtered_views"]) < 1e-5


def test_monte_mc_program_writes_reference_files(tmp_path):
    # a 200^3 label volume like the reference's: water cylinder, Ca rods
    k, j, i = np.ogrid[0:200, 0:200, 0:200]
    x, y = (i + 0.5) / 10 - 10, (j + 0.5) / 10 - 10
    lab = np.zeros((200, 200, 200), np.uint8)
    lab[np.broadcast_to(x * x + y * y <= 64, lab.shape)] = 1
    lab[np.broadcast_to((x - 5) ** 2 + y ** 2 <= 2.25, lab.shape)] = 2
    lab.tofile(tmp_path / "cyu8_2.raw")
    x = golden("xcom")
    for name, t in (("xcom2.csv", x["water"]), ("Ca.csv", x["ca"])):
        with open(tmp_path / name, "w") as f:
            for r in range(1, 201):
                f.write("%.6g,%.6g,%.6g,%.9g\r\n" % tuple(t[:, r]))
    per, views = 20, 4
    subprocess.run([os.path.join(PROG, "monte_mc"), "--per", str(per), "--views", str(views)],
                   cwd=tmp_path, check=True, capture_output=True)
    n = views * 325 * 325
    p0 = np.fromfile(tmp_path / "proj325_teth0pmma8etim2.raw", np.int32)
    p5 = np.fromfile(tmp_path / "proj325_teth5pmma8etim2.raw", np.int32)
    m0 = np.fromfile(tmp_path / "map325_teth0pmma8etim2.raw", np.float32)
    assert p0.size == n and p5.size == n and m0.size == n
    assert p0.min() >= 1 and p0.max() <= per and np.all(p5 >= p0)
    want = (-np.log(p0.astype(np.float64)) + np.float64(np.float32(np.log(per)))).astype(np.float32)
    assert np.array_equal(m0, want)
    # the field outside the cylinder shadow is unattenuated: all histories reach it
    assert np.median(p0.reshape(views, 325, 325)[:, :5, :]) == per


def test_monte_fbp2_program_matches_fbp2(tmp_path):
    gold = golden("fbp2")
    proj = fdk_projections(360, 65, 1, int(gold["seed"])).reshape(360, 65)
    proj.tofile(tmp_path / "map5_20_2e5.raw")
    subprocess.run([os.path.join(PROG, "monte_fbp2")], cwd=tmp_path, check=True,
                   capture_output=True)
    img = np.fromfile(tmp_path / "projection_test\\testxyo2e5.raw", np.float32).reshape(256, 256)
    filt = np.fromfile(tmp_path / "projection_test\\outproj2e5.raw", np.float32).reshape(360, 65)
    assert np.array_equal(img, gold["image"])
    assert np.array_equal(filt, gold["filtered"])
