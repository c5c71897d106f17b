"""Generate the golden fixtures in tests/golden/ by running the reference's
own CPU programs (compiled unmodified by oracle/build_ref.sh) on seeded
synthetic inputs.  Run in the container that holds the reference tree:

    oracle/build_ref.sh && python tests/golden/make_golden.py [--only NAME]

Fixtures (all small; inputs are regenerated from their seeds by
tests/golden/inputs.py):
  fdk65.npz     recon/bp3d20.cpp on fdk_projections(360,65,65,seed=1065):
                xy slab [256][256][125:130], 4 filtered views
  fdk325.npz    recon/bp3d20_325.cpp on fdk_projections(360,325,325,seed=1325):
                xy slab, filtered rows of 4 views
  fbp2.npz      recon/fbp2.cpp on fdk_projections(360,65,1,seed=2065):
                its filtered projections and 256x256 image
  cbct_real2.npz  monte_cpp/CBCT_real2.cpp (10^7 histories from pixel
                (32,32) at 140 keV through the spher01.raw water sphere):
                the 65x65 Compton-scatter tally it writes
  xcom.npz      monte_cpp/xcom2.csv (water) and monte_cpp/Ca.csv parsed into
                [4][201] float32 tables indexed by keV (coh, incoh, photo, total)
"""
import argparse
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, HERE)
from inputs import fdk_projections  # noqa: E402

# the reference tree: MONTE_REFERENCE, else a "reference" directory beside
# the repository
REF = os.environ.get("MONTE_REFERENCE", os.path.join(os.path.dirname(REPO), "reference"))
BIN = os.path.join(REPO, "oracle", "_ref")


def run(binary, cwd):
    subprocess.run([os.path.join(BIN, binary)], cwd=cwd, check=True,
                   stdout=subprocess.DEVNULL)


def fdk(name, n, seed, binary, in_name, out_stem, view_ids, row_ids):
    proj = fdk_projections(360, n, n, seed)
    with tempfile.TemporaryDirectory() as tmp:
        proj.tofile(os.path.join(tmp, in_name))
        run(binary, tmp)
        xy = np.fromfile(os.path.join(tmp, "CBCTrecon\\xy" + out_stem + ".raw"), np.float32)
        zy = np.fromfile(os.path.join(tmp, "CBCTrecon\\zy" + out_stem + ".raw"), np.float32)
        filt = np.fromfile(os.path.join(tmp, "CBCTrecon\\map" + out_stem + ".raw"), np.float32)
    xy = xy.reshape(256, 256, 256)
    zy = zy.reshape(256, 256, 256)
    filt = filt.reshape(360, n, n)
    assert np.array_equal(xy.transpose(2, 1, 0), zy), "zy is not the transpose of xy"
    nz = np.nonzero(np.any(xy != 0, axis=(0, 1)))[0]
    assert nz.min() >= 125 and nz.max() < 130, nz
    out = dict(seed=np.int64(seed), xy_slab=np.ascontiguousarray(xy[:, :, 125:130]),
               view_ids=np.array(view_ids), row_ids=np.array(row_ids))
    if row_ids is None or len(row_ids) == 0:
        out["filtered_views"] = filt[view_ids]
    else:
        out["filtered_rows"] = filt[view_ids][:, row_ids, :]
    np.savez(os.path.join(HERE, name + ".npz"), **out)
    print(name, "xy slab norm", float(np.linalg.norm(out["xy_slab"])))


def fbp2():
    proj = fdk_projections(360, 65, 1, 2065).reshape(360, 65)
    with tempfile.TemporaryDirectory() as tmp:
        proj.tofile(os.path.join(tmp, "map5_20_2e5.raw"))
        run("fbp2", tmp)
        filt = np.fromfile(os.path.join(tmp, "projection_test\\outproj2e5.raw"), np.float32)
        img = np.fromfile(os.path.join(tmp, "projection_test\\testxyo2e5.raw"), np.float32)
    np.savez(os.path.join(HERE, "fbp2.npz"), seed=np.int64(2065), filtered=filt.reshape(360, 65),
             image=img.reshape(256, 256))
    print("fbp2 image norm", float(np.linalg.norm(img)))


def parse_xcom(path):
    """BOM/CRLF-tolerant parse of an XCOM csv: row r (1-based) -> index r
    (monte_cpp/CBCT_real2.cpp:633-668); index 0 repeats row 1."""
    with open(path, "rb") as f:
        text = f.read().decode("utf-8-sig")
    rows = [ln for ln in text.replace("\r", "").split("\n") if ln.strip()]
    tab = np.zeros((4, 201), np.float32)
    for r, ln in enumerate(rows, start=1):
        vals = [float(x) for x in ln.split(",")[:4]]
        tab[:, r] = vals
    tab[:, 0] = tab[:, 1]
    return tab


def xcom():
    water = parse_xcom(os.path.join(REF, "monte_cpp", "xcom2.csv"))
    ca = parse_xcom(os.path.join(REF, "monte_cpp", "Ca.csv"))
    np.savez(os.path.join(HERE, "xcom.npz"), water=water, ca=ca)
    print("xcom water mu(60)=%g ca mu(60)=%g" % (water[3, 60], ca[3, 60]))


def cbct_real2():
    with tempfile.TemporaryDirectory() as tmp:
        run("make_image01", tmp)  # writes spher01.raw
        for f in ("xcom2.csv", "Ca.csv"):
            shutil.copy(os.path.join(REF, "monte_cpp", f), tmp)
        # The spectrum tables are not in the reference tree; their values are
        # unused because the program forces 140 keV (CBCT_real2.cpp:188,219),
        # but readcsv needs 250 parsable rows (:664-667).
        for f in ("125kv_al2mm.csv", "125kv_al10mm.csv"):
            with open(os.path.join(tmp, f), "w") as fh:
                for i in range(250):
                    fh.write("%d,0,0,%.6f\n" % (i, (i + 1) / 250.0))
        log = subprocess.run([os.path.join(BIN, "CBCT_real2")], cwd=tmp, check=True,
                             capture_output=True, text=True).stdout
        img = np.fromfile(os.path.join(tmp, "CBCTtest3\\monte005.raw"), np.int32).reshape(65, 65)
    print("CBCT_real2 tally sum", int(img.sum()))
    np.savez(os.path.join(HERE, "cbct_real2.npz"), image=img, histories=np.int64(10**7),
             log=np.array(log[-2000:]))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", default=None)
    a = ap.parse_args()
    jobs = {
        "xcom": xcom,
        "fdk65": lambda: fdk("fdk65", 65, 1065, "bp3d20", "mapg_0_20000h2oCa.raw",
                             "2mh20kyu2", [0, 97, 201, 359], []),
        "fdk325": lambda: fdk("fdk325", 325, 1325, "bp3d20_325", "mapg325_0_2tca.raw",
                              "ca0_2t", [0, 97, 201, 359], [0, 100, 162, 324]),
        "fbp2": fbp2,
        "cbct_real2": cbct_real2,
    }
    for k, fn in jobs.items():
        if a.only is None or a.only == k:
            fn()


if __name__ == "__main__":
    main()
