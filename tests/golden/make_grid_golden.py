"""Regenerate the grid golden fixtures with the reference's own pre-processor.

Runs the reference's 01_pre_processor/grid.py (unchanged, in a scratch
directory) on a grid.input per case, then lib_setgrid.setgrid and
lib_preprocessing.grid_preprocessing_data on its grid.dat, and stores the
resulting grid.dat / grid.bin texts here.  tests/test_grid_golden.py checks
that leswht_gb300.gridgen reproduces both files byte for byte.

Only runs where the reference checkout exists (pass its path as argv[1]);
the committed fixtures are what the tests use.
"""
from __future__ import annotations

import math
import os
import shutil
import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent

# name: (N, L, segments per direction (dir, ci, cf, ii, if, opt, f1, f2), (xprdic, zprdic))
CASES = {
    "channel_16x16x8": (
        (17, 17, 9), (4.0 * math.pi, 2.0, 4.0 * math.pi / 3.0),
        [("X", 0.0, 4.0 * math.pi, 1, 17, "U", 0.0, 0.0),
         ("Y", -1.0, 1.0, 1, 17, "H", 0.5, 2.75),
         ("Z", 0.0, 4.0 * math.pi / 3.0, 1, 9, "U", 0.0, 0.0)],
        (True, True)),
    "channel_64x64x64": (
        (65, 65, 65), (4.0 * math.pi, 2.0, 4.0 * math.pi / 3.0),
        [("X", 0.0, 4.0 * math.pi, 1, 65, "U", 0.0, 0.0),
         ("Y", -1.0, 1.0, 1, 65, "H", 0.5, 2.75),
         ("Z", 0.0, 4.0 * math.pi / 3.0, 1, 65, "U", 0.0, 0.0)],
        (True, True)),
    "cylinder_32x24x4": (
        (33, 25, 5), (30.0, 20.0, math.pi),
        [("X", -10.0, -1.0, 1, 9, "G", 0.0, 1.2),
         ("X", -1.0, 1.0, 9, 21, "U", 0.0, 0.0),
         ("X", 1.0, 20.0, 21, 33, "G", 1.0, 1.15),
         ("Y", -10.0, 10.0, 1, 25, "H", 0.5, 2.0),
         ("Z", 0.0, math.pi, 1, 5, "U", 0.0, 0.0)],
        (False, True)),
}


def grid_input_text(n, l, segs) -> str:
    out = ["N_x N_y N_z L_x L_y L_z\n",
           "%d %d %d %r %r %r\n" % (n[0], n[1], n[2], l[0], l[1], l[2]),
           "Dir. Coord_i Coord_f Index_i Index_f Grid_opt Factor1 Factor2\n"]
    for s in segs:
        out.append("%s %r %r %d %d %s %r %r\n" % s)
    out.append("----- end\n")
    out.append("Debugging Options\n")
    out.append("Midpoints XY YZ ZX dx dy dz\n")
    out.append("OFF OFF OFF OFF OFF OFF OFF\n")
    return "".join(out)


def main(ref_root: str) -> None:
    pre = Path(ref_root) / "01_pre_processor"
    sys.path.insert(0, str(pre))
    from lib import lib_preprocessing, lib_setgrid  # noqa: E402  (reference modules)
    for name, (n, l, segs, (xp, zp)) in CASES.items():
        with tempfile.TemporaryDirectory() as tmp:
            work = Path(tmp) / "pre"
            (Path(tmp) / "output" / "grid").mkdir(parents=True)
            work.mkdir()
            (work / "grid.input").write_text(grid_input_text(n, l, segs))
            subprocess.run([sys.executable, str(pre / "grid.py")], cwd=work, check=True,
                           stdout=subprocess.DEVNULL)
            cwd = os.getcwd()
            os.chdir(work)
            try:
                g = lib_setgrid.setgrid("../output/grid/grid.dat", "ON" if xp else "OFF", "OFF",
                                        "ON" if zp else "OFF")
                lib_preprocessing.grid_preprocessing_data(g)
            finally:
                os.chdir(cwd)
            shutil.copy(Path(tmp) / "output" / "grid" / "grid.dat", HERE / f"{name}.grid.dat")
            shutil.copy(Path(tmp) / "output" / "grid" / "grid.bin", HERE / f"{name}.grid.bin")
        print("wrote", name)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_grid_golden.py <path of the LESwHT checkout>")
    main(sys.argv[1])
