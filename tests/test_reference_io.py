"""The boundary files against the reference's own files and readers (CPU).

* The reference's 02_solver/settings.input and boundary.input, as shipped
  (committed verbatim under tests/golden/ by make_io_golden.py), read by the
  compiled driver's readsettings / readbcs restatement: every value a Fortran
  list-directed read of those files gives, the header rows and the trailing
  example rows and free text skipped, readbcs's periodic override applied.
* Field and fav files written by this library's writers, read by the
  reference's post-processor (post_inst.py read_inst_field, post_avg.py
  read_avg_field) when the fixtures were made: the files written here today
  are the same bytes, and the arrays the reference's readers returned hold
  the written values in the right cells.
"""
import hashlib
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import leswht_gb300
from leswht_gb300 import cases, fileio

GOLD = Path(__file__).resolve().parent / "golden"

import importlib.util as _ilu  # noqa: E402
_spec = _ilu.spec_from_file_location("make_io_golden", GOLD / "make_io_golden.py")
gold = _ilu.module_from_spec(_spec)
_spec.loader.exec_module(gold)


def _sha(path):
    with open(path, "rb") as f:
        return hashlib.sha256(f.read()).hexdigest()


def _dry_run(sdir):
    exe = leswht_gb300.exec_path()
    out = subprocess.run([str(exe), "--dry-run"], cwd=sdir, capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    d = {}
    for line in out.stdout.splitlines():
        k, *v = line.split()
        d[k] = v
    return d


# What readsettings (misc_init.f90:19-92) and readbcs (:95-158) read from the
# reference's shipped input files.
REF_SETTINGS = dict(
    re=180.0, pr=0.71, gr=0.0, grdir=2, tflu_i=0.0, tsol_i=0.0,
    ireset=1, iread=0, iavg=1, ipzero=0, eps_ptr=6.0, udrv_i=1.0,
    nend=999999, nprint=10000, npriavg=50000, npin=1,
    tend=200.0, ptb_tst=4.0, avg_tst=20.0,
    idtopt=1, dt_size=0.005, cflfac=1.0,
    resid1=1.0e-6, nlev=5, nbli=3, ioldv=0, mgitr=500, imgsor=170, wwsor=1.8,
    iles=1, insmdl=1, itemdl=0, idvmon=1, csgsts=0.025, csgshf=0.003, filter=3,
    ibmon=1, masson=1, imovingon=0, ihtrans=1, idecomp=1)
REF_BOUNDARY = dict(
    bc_ybtm=0, bc_ytop=0, bc_t_ybtm=0, bc_t_ytop=0, val_t_ybtm=0.0, val_t_ytop=0.0,
    bc_t_zbtm=1, bc_t_ztop=1, val_t_zbtm=0.0, val_t_ztop=0.0, ich=2, iconjg=1)


def test_exec_reads_the_reference_input_files(tmp_path):
    c = cases.channel(16, 16, 8)
    sdir = fileio.write_case_dir(str(tmp_path), c, nend=1)
    for f in ("settings", "boundary"):
        shutil.copyfile(GOLD / f"ref_{f}.input", os.path.join(sdir, f"{f}.input"))
    d = _dry_run(sdir)
    for k, v in {**REF_SETTINGS, **REF_BOUNDARY}.items():
        got = d[k][0]
        assert (int(got) if isinstance(v, int) else float(got)) == v, k
    # FILES: the quoted paths; TRACE NTR: 0 tracking points, every step; the
    # "10 10 10" row and the descriptions after it are not read
    assert d["gridfile"] == ["../output/grid/grid.bin"]
    assert d["prev_fld"] == ["../output/field/fld000000"]
    assert d["trace"] == ["0", "1"]
    # readbcs: a periodic direction's momentum flags become 4 (the case's
    # ibmpre_prdic.bin has x and z periodic)
    assert (d["xprdic"], d["zprdic"]) == (["1"], ["1"])
    assert (d["bc_zbtm"], d["bc_ztop"]) == (["4"], ["4"])


def test_exec_reads_tracking_points(tmp_path):
    c = cases.channel(16, 16, 8)
    sdir = fileio.write_case_dir(str(tmp_path), c, nend=1)
    text = open(os.path.join(sdir, "settings.input")).read().splitlines()
    assert text[-2].startswith("TRACE")
    text[-1] = "2       5"
    text += ["5    3   4     first point", "10   6   8", "10      10      10"]
    with open(os.path.join(sdir, "settings.input"), "w") as f:
        f.write("\n".join(text) + "\n")
    d = _dry_run(sdir)
    assert d["trace"] == ["2", "5", "5", "3", "4", "10", "6", "8"]


def test_exec_rejects_truncated_settings(tmp_path):
    c = cases.channel(16, 16, 8)
    sdir = fileio.write_case_dir(str(tmp_path), c, nend=1)
    text = open(os.path.join(sdir, "settings.input")).read().splitlines()
    with open(os.path.join(sdir, "settings.input"), "w") as f:
        f.write("\n".join(text[:9]) + "\n")
    out = subprocess.run([str(leswht_gb300.exec_path()), "--dry-run"], cwd=sdir, capture_output=True, text=True,
                         timeout=120)
    assert out.returncode != 0 and "unexpected end of file" in out.stderr


@pytest.mark.parametrize("name", sorted(gold.golden_cases()))
def test_reference_post_processor_reads_our_field_file(tmp_path, name):
    case = gold.golden_cases()[name]
    s, g = case.settings, case.grid
    f = gold.seeded_fields(case, gold.SEED)
    path = str(tmp_path / "fld0000042")
    fileio.write_field(path, s, g, f, 42, 420, 2.5, 0.004)
    ref = np.load(GOLD / f"post_inst_{name}.npz")
    assert _sha(path) == str(ref["file_sha256"])
    assert list(ref["scalars"]) == [s["re"], s["pr"], s["gr"]]
    n1, n2, n3, n1m, n2m, n3m = g.n1, g.n2, g.n3, g.n1m, g.n2m, g.n3m
    # the reference's arrays are (i, j, k); ours (k, j, i).  Compare every
    # cell the records hold, away from the planes its periodic copies rewrite
    T_ = lambda a: np.transpose(a, (2, 1, 0))   # noqa: E731
    assert np.array_equal(ref["U"][1:n1, 0:n2 + 1, 1:n3], T_(f["u"][1:n3, 0:n2 + 1, 1:n1]))
    assert np.array_equal(ref["V"][1:n1, 1:n2 + 1, 1:n3], T_(f["v"][1:n3, 1:n2 + 1, 1:n1]))
    assert np.array_equal(ref["W"][1:n1, 0:n2 + 1, 1:n3], T_(f["w"][1:n3, 0:n2 + 1, 1:n1]))
    assert np.array_equal(ref["P"][1:n1m + 1, 1:n2m + 1, 1:n3m + 1], T_(f["p"][1:n3m + 1, 1:n2m + 1, 1:n1m + 1]))
    if s.get("ihtrans", 0) == 1:
        assert np.array_equal(ref["T"][1:n1m + 1, 1:n2m + 1, 1:n3m + 1],
                              T_(f["t"][1:n3m + 1, 1:n2m + 1, 1:n1m + 1]))


@pytest.mark.parametrize("name", sorted(gold.golden_cases()))
def test_reference_post_processor_reads_our_fav_file(tmp_path, name):
    case = gold.golden_cases()[name]
    s, g = case.settings, case.grid
    ih = int(s.get("ihtrans", 0))
    sums, t0, t1, h0, h1 = gold.seeded_fav(case, gold.SEED)
    path = str(tmp_path / "fav0000003-0000018")
    fileio.write_fav(path, s["re"], (g.n1m, g.n2m, g.n3m), sums, t0, t1, h0, h1, ih)
    ref = np.load(GOLD / f"post_avg_{name}.npz")
    assert _sha(path) == str(ref["file_sha256"])
    assert (float(ref["scalar_TIMEINIT"]), float(ref["scalar_TIMEEND"])) == (t0, t1)
    assert (float(ref["scalar_IHISTINIT"]), float(ref["scalar_IHISTEND"])) == (h0, h1)
    assert float(ref["scalar_Re"]) == s["re"]
    # our reader and the reference's agree cell for cell (the reference
    # divides the sums by the window, TIMEEND - TIMEINIT)
    ours = fileio.read_fav(path, ih)
    win = t1 - t0
    keys = {"uavg": "UAVG", "vavg": "VAVG", "wavg": "WAVG", "uiujavg": "UIUJAVG", "pavg": "PAVG",
            "p2avg": "P2AVG", "voravg": "VORAVG", "vor2avg": "VOR2AVG", "ssavg": "SSAVG"}
    if ih == 1:
        keys.update(tavg="TAVG", t2avg="T2AVG")
    n1m, n2m, n3m = g.n1m, g.n2m, g.n3m
    for k, rk in keys.items():
        a = ours[k] / win
        r = ref[rk]
        if a.ndim == 4:
            r = r[:, 1:n1m + 1, 1:n2m + 1, 1:n3m + 1]
            assert np.array_equal(r, np.transpose(a, (0, 3, 2, 1))), k
        else:
            r = r[1:n1m + 1, 1:n2m + 1, 1:n3m + 1]
            assert np.array_equal(r, np.transpose(a, (2, 1, 0))), k
