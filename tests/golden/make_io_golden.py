"""Regenerate the on-disk-format golden fixtures with the reference's own code.

Takes the path of a LESwHT checkout (argv[1]) and writes into this folder:

* ref_settings.input, ref_boundary.input -- the solver's two text inputs
  exactly as the reference ships them (02_solver/), with the header rows,
  the free-text parameter descriptions and the tracking-point example rows
  that readsettings / readbcs must skip; tests/test_reference_io.py runs the
  compiled driver's readers on them.
* post_inst_<case>.npz -- a field file written by leswht_gb300.fileio
  (the writer whose layout lesgpu_exec's field files match byte for byte)
  from seeded values, read back by the reference's post-processor
  (03_post_processor/inst/post_inst.py read_inst_field): the arrays it
  returned.
* post_avg_<case>.npz -- likewise a fav file from fileio.write_fav read by
  03_post_processor/avg/post_avg.py read_avg_field.

The test regenerates each file from the same seed and checks that the
post-processor's arrays equal the values written, so the files this library
writes are the files the reference's own readers expect.  Nothing here runs
during the tests.
"""
from __future__ import annotations

import contextlib
import hashlib
import io
import os
import shutil
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

import numpy as np  # noqa: E402

from leswht_gb300 import cases, fileio  # noqa: E402

SEED = 20261204


def golden_cases():
    """name -> case; the values written are seeded, not the case's fields."""
    return {
        "channel_8x6x4": cases.channel(8, 6, 4),
        "cylinder_16x12x4": cases.cylinder(16, 12, 4),
    }


def seeded_fields(case, seed):
    rng = np.random.default_rng(seed)
    return {k: rng.standard_normal(case.grid.shape) for k in ("u", "v", "w", "p", "t")}


def seeded_fav(case, seed):
    g = case.grid
    ih = int(case.settings.get("ihtrans", 0))
    nval = sum(fileio.FAV_COUNTS[:11 if ih == 1 else 9])
    rng = np.random.default_rng(seed + 1)
    return rng.standard_normal(nval * g.n1m * g.n2m * g.n3m), 0.25, 1.75, 3, 18


def sha256(path):
    with open(path, "rb") as f:
        return hashlib.sha256(f.read()).hexdigest()


def _grid_data(mod, g):
    gd = mod.GridData()
    gd.N1, gd.N2, gd.N3 = g.n1, g.n2, g.n3
    gd.N1M, gd.N2M, gd.N3M = g.n1m, g.n2m, g.n3m
    return gd


def main(ref: str) -> None:
    ref = Path(ref)
    for f in ("settings", "boundary"):
        shutil.copyfile(ref / "02_solver" / f"{f}.input", HERE / f"ref_{f}.input")
    sys.path.insert(0, str(ref / "03_post_processor" / "inst"))
    sys.path.insert(0, str(ref / "03_post_processor" / "avg"))
    import post_avg  # noqa: E402
    import post_inst  # noqa: E402
    for name, case in golden_cases().items():
        s, g = case.settings, case.grid
        ih = int(s.get("ihtrans", 0))
        with tempfile.TemporaryDirectory() as tmp:
            fileio.write_field(os.path.join(tmp, "fld0000042"), s, g, seeded_fields(case, SEED), 42, 420, 2.5, 0.004)
            with contextlib.redirect_stdout(io.StringIO()):
                U, V, W, P, T, *rest = post_inst.read_inst_field("fld0000042", _grid_data(post_inst, g), ih,
                                                                 int(s["xprdic"]), int(s["zprdic"]), field_dir=tmp)
            np.savez_compressed(HERE / f"post_inst_{name}.npz", U=U, V=V, W=W, P=P, T=T,
                                scalars=np.array([float(x) for x in rest[:3]]),
                                file_sha256=np.array(sha256(os.path.join(tmp, "fld0000042"))))
            sums, t0, t1, h0, h1 = seeded_fav(case, SEED)
            fileio.write_fav(os.path.join(tmp, "fav0000003-0000018"), s["re"], (g.n1m, g.n2m, g.n3m), sums,
                             t0, t1, h0, h1, ih)
            with contextlib.redirect_stdout(io.StringIO()):
                d = post_avg.read_avg_field("fav0000003-0000018", _grid_data(post_avg, g), ih, field_dir=tmp)
            arrays = {}
            for k, v in d.items():
                if isinstance(v, list):
                    arrays[k] = np.stack(v)
                elif isinstance(v, np.ndarray):
                    arrays[k] = v
                else:
                    arrays["scalar_" + k] = np.array(float(v))
            arrays["file_sha256"] = np.array(sha256(os.path.join(tmp, "fav0000003-0000018")))
            np.savez_compressed(HERE / f"post_avg_{name}.npz", **arrays)
        print("wrote", name)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_io_golden.py <path of the LESwHT checkout>")
    main(sys.argv[1])
