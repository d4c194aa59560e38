"""Generate the golden fixtures in this folder from the jif3D reference.

* box_terms.json  -- g_z and the 9 FTG prism terms of the reference's own
  Gravity/BasicGravElements.cpp (compiled unmodified by ``make -C oracle ref``)
  at seeded random and degenerate station / prism configurations.
* simpeg_mag.json -- the SimPEG comparison values that the reference's
  Magnetics/test_MagneticCalculation.cpp:164-217 checks against
  (jif3D/magx.simpeg, magy, magz, magt: Bx, By, Bz, TFA in nT).
* tutorial5_gravdata.nc, tutorial5_magdata.nc -- the gravity and total-field
  magnetic data files of jif3D's Tutorial 5 (netCDF-4 / HDF5 files written by
  jif3D), copied unchanged, and netcdf_tutorial.json -- the values the
  tutorial notebook printed after reading magdata.nc with netCDF4 (station
  spacing and the range of MeasPosX / MeasPosY), taken from the notebook's
  stored output.

Run where the reference sources exist:
    python tests/golden/make_golden.py <path/to/jif3D>
Machines without the reference tree run the tests on the committed files.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def box_cases(rng):
    cases = []
    # known-answer configurations of Gravity/test_ScalarCalculation.cpp:32-64
    cases += [
        [0.0, 0.0, 0.0, -10.0, -10.0, -10.0, 20.0, 20.0, 20.0],
        [0.0, 0.0, -10.0, -10.0, -10.0, -10.0, 20.0, 20.0, 20.0],
        [0.0, 0.0, 10.0, -10.0, -10.0, -10.0, 20.0, 20.0, 20.0],
        [10.0, 10.0, 0.0, 0.0, 0.0, 0.0, 20.0, 20.0, 20.0],
        [1e5, 10.0, 10.0, -10.0, -10.0, -10.0, 20.0, 20.0, 20.0],
        [100.0, 100.0, 10.0, -10.0, -10.0, -10.0, 20.0, 20.0, 20.0],
        [0.0, 0.0, 0.0, -1e6, -1e6, -1e6, 2e6, 2e6, 2e6],
        [9.0, 8.0, -0.1, 0.0, 0.0, 0.0, 20.0, 20.0, 20.0],
    ]
    # station on a corner, an edge and a face of the prism
    cases += [
        [0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 10.0, 10.0, 10.0],
        [5.0, 0.0, 0.0, 0.0, 0.0, 0.0, 10.0, 10.0, 10.0],
        [5.0, 5.0, 0.0, 0.0, 0.0, 0.0, 10.0, 10.0, 10.0],
        [0.0, 5.0, -3.0, 0.0, 0.0, 0.0, 10.0, 10.0, 10.0],
        [10.0, 10.0, 10.0, 0.0, 0.0, 0.0, 10.0, 10.0, 10.0],
    ]
    for t in range(300):
        m = rng.uniform(-3000, 3000, 3)
        c = rng.uniform(-3000, 3000, 3)
        s = rng.uniform(1, 400, 3)
        if t % 4 == 0:
            m, c, s = np.round(m), np.round(c), np.round(s)
        if t % 7 == 0:
            m[2] = -abs(m[2]) - 1.0
            c[2] = abs(c[2])
        cases.append([float(v) for v in np.concatenate([m, c, s])])
    return cases


def main():
    if len(sys.argv) < 2:
        raise SystemExit("usage: make_golden.py <jif3D source tree>")
    ref_root = sys.argv[1]
    os.environ["JIF3D_REF"] = ref_root
    from oracle import oracle as O
    O.build()
    R = O.ref_lib()
    if R is None:
        raise SystemExit("reference box-term library was not built")
    rng = np.random.default_rng(20241203)
    out = []
    for args in box_cases(rng):
        t = np.zeros(9)
        R.ref_tensor_box(*args, t.ctypes.data_as(O._P))
        out.append({"args": args, "gz": R.ref_grav_box(*args), "tensor": t.tolist()})
    with open(os.path.join(HERE, "box_terms.json"), "w") as f:
        json.dump({"source": "jif3D Gravity/BasicGravElements.cpp (CalcGravBoxTerm, "
                             "CalcTensorBoxTerm)", "cases": out}, f)
    sim = {}
    for comp in ("x", "y", "z", "t"):
        with open(os.path.join(ref_root, f"mag{comp}.simpeg")) as f:
            sim[comp] = [float(v) for v in f.read().split()]
    sim["setup"] = {"ncells": 10, "xsize": 2.0, "ysize": 4.0, "zsize": 0.5, "chi": 0.2,
                    "inclination_deg": 15.0, "declination_deg": 10.0, "fs": 50000.0,
                    "stations": "x = -20 + i/5 (i < 200), y = 10, z = -1",
                    "origin": "(-widthx/2, -widthy/2, 0)",
                    "source": "jif3D Magnetics/test_MagneticCalculation.cpp:110-217"}
    with open(os.path.join(HERE, "simpeg_mag.json"), "w") as f:
        json.dump(sim, f)
    print("wrote", len(out), "box cases and", len(sim["x"]), "SimPEG stations")
    tutorial(os.path.join(ref_root, "Tutorial", "Tutorial5"))


def tutorial(folder):
    import hashlib
    import re
    import shutil
    meta = {"source": "jif3D Tutorial/Tutorial5 (gravdata.nc, magdata.nc, Tutorial5.ipynb)",
            "files": {}}
    for name in ("gravdata.nc", "magdata.nc"):
        dst = os.path.join(HERE, "tutorial5_" + name)
        shutil.copyfile(os.path.join(folder, name), dst)
        with open(dst, "rb") as f:
            meta["files"][os.path.basename(dst)] = hashlib.sha256(f.read()).hexdigest()
    with open(os.path.join(folder, "Tutorial5.ipynb")) as f:
        nb = json.load(f)
    printed = None
    for cell in nb["cells"]:
        src = "".join(cell.get("source", []))
        if 'Dataset("magdata.nc"' in src:
            printed = "".join("".join(o.get("text", [])) for o in cell.get("outputs", []))
    if printed is None:
        raise SystemExit("notebook cell reading magdata.nc not found")
    keys = {"Data spacing": "spacing", "Minimum x": "min_x", "Maximum x": "max_x",
            "Minimum y": "min_y", "Maximum y": "max_y"}
    meta["magdata_printed"] = {}
    for line in printed.splitlines():
        m = re.match(r"\s*([A-Za-z ]+):\s*(\S+)", line)
        if m and m.group(1).strip() in keys:
            meta["magdata_printed"][keys[m.group(1).strip()]] = m.group(2)
    with open(os.path.join(HERE, "netcdf_tutorial.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print("copied the Tutorial 5 data files;", meta["magdata_printed"])


if __name__ == "__main__":
    main()
