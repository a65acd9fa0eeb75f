"""The compiled driver lesgpu_exec (the counterpart of the reference's
solver_exec) run on case directories: its field files, history files and
field-average files equal what the same case gives through the Python host
driver started from the same stored field (bitwise for the fields and the
averages, and character for character for the formatted histories)."""
import os
import subprocess

import numpy as np
import pytest

import leswht_gb300
from leswht_gb300 import abi, cases, fileio

pytestmark = pytest.mark.gpu

FMT5 = "%13.5f%15.7E%15.7E%15.7E%15.7E"
FMT7 = "%13.5f%15.7E%15.7E%15.7E%15.7E%15.7E%15.7E"


def run_exec(sdir):
    out = subprocess.run([str(leswht_gb300.exec_path())], cwd=sdir, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stdout + out.stderr
    return out.stdout


def restart_case(root, c, s):
    """The case as prefld leaves it after reading root's fld0000000."""
    r = fileio.read_field(os.path.join(root, "output", "field", "fld0000000"), c.grid, s["ihtrans"], s["tsol_i"])
    U, V, W, P, T = cases.prefld_apply(s, c.grid, r["u"], r["v"], r["w"], r["p"], r["t"])
    if s["ihtrans"] != 1:
        T = np.full(c.grid.shape, float(s["tsol_i"]))
    return cases.Case(c.name, s, c.grid, c.grid_dat, c.grid_bin, dict(u=U, v=V, w=W, p=P, t=T),
                      time=r["time"], dt=r["dt"], ihist=r["ihist"], m=r["m"], ibm=c.ibm)


def check_field(path, c, fields, rep, ihtrans):
    r = fileio.read_field(path, c.grid, ihtrans)
    g = c.grid
    n1, n2, n3 = g.n1, g.n2, g.n3
    sl = {"u": np.s_[0:n3 + 1, 0:n2 + 1, 1:n1 + 1], "v": np.s_[0:n3 + 1, 1:n2 + 1, 0:n1 + 1],
          "w": np.s_[1:n3 + 1, 0:n2 + 1, 0:n1 + 1], "p": np.s_[1:n3, 1:n2, 1:n1]}
    if ihtrans == 1:
        sl["t"] = np.s_[1:n3, 1:n2, 1:n1]
    for k, q in sl.items():
        assert np.array_equal(r[k][q], fields[k][q]), (path, k)
    assert (r["m"], r["time"], r["dt"]) == (rep["m"], rep["time"], rep["dt"])
    # byte for byte the file fileio.write_field makes, whose layout the
    # reference's post-processor reads (tests/test_reference_io.py)
    want = path + ".want"
    fileio.write_field(want, c.settings, g, fields, r["ihist"], rep["m"], rep["time"], rep["dt"])
    with open(path, "rb") as a, open(want, "rb") as b:
        assert a.read() == b.read(), path
    os.unlink(want)


def lines(path):
    with open(path) as f:
        return f.read().splitlines()


@pytest.fixture(autouse=True)
def _reproducible_across_processes(monkeypatch):
    # the driver and this process must pick the same ADI lane counts
    monkeypatch.setenv("LESGPU_AUTOTUNE", "0")


def test_exec_channel_fields_history_and_averages(tmp_path):
    c = cases.channel(32, 32, 16)
    c.settings.update(iavg=1, avg_tst=0.0, npriavg=4)
    root = str(tmp_path)
    sdir = fileio.write_case_dir(root, c, nend=6, nprint=3, npin=1)
    run_exec(sdir)
    s = dict(c.settings); s.update(iread=1, ireset=0, nend=6, nprint=3, npin=1)
    rc = restart_case(root, c, s)
    sol = leswht_gb300.gpu_solver(rc)
    reps, avgs = [], []
    for n in range(1, 7):
        rep = sol.step()
        reps.append(rep)
        if n % 3 == 0:
            check_field(os.path.join(root, "output", "field", "fld%07d" % n), rc, sol.fields(), rep, 1)
        if n in (4, 6):
            avgs.append(sol.averages(reset=True)[0])
    hist = lines(os.path.join(root, "output", "ftr", "fhist.dat"))
    assert hist == [FMT5 % (r["time"], r["dt"], r["cflmax"], r["dvmax"], r["qmmax"]) for r in reps]
    cmfr = lines(os.path.join(root, "output", "ftr", "fcmfr.dat"))
    assert len(cmfr) == 6
    assert [float(x) for x in cmfr[0].split()[1:4]] == pytest.approx([reps[0]["qflux"], reps[0]["ubulk"],
                                                                       reps[0]["pmiavg"]], rel=1e-6)
    ftemp = lines(os.path.join(root, "output", "ftr", "ftemp.dat"))
    assert ftemp[2].split()[1] == ("%15.7E" % reps[2]["tbulk_fluid"]).strip()
    assert len(lines(os.path.join(root, "output", "ftr", "ftime.dat"))) == 6
    fav = sorted(os.listdir(os.path.join(root, "output", "field_avg")))
    assert "fav0000001-0000004" in fav and "fav0000004-0000006" in fav
    assert lines(os.path.join(root, "output", "field_avg", "fav_manifest.dat")) == ["fav0000001-0000004",
                                                                                   "fav0000004-0000006"]
    for name, want in (("fav0000001-0000004", avgs[0]), ("fav0000004-0000006", avgs[1])):
        f = fileio.read_fav(os.path.join(root, "output", "field_avg", name), 1)
        assert np.array_equal(f["uavg"], want["uavg"]) and np.array_equal(f["t2avg"], want["t2avg"])
        assert np.array_equal(f["vor2avg"][5], want["wzwz"]) and np.array_equal(f["uiujavg"][1], want["uv"])
        # byte for byte the file fileio.write_fav makes from the same sums
        fpath = os.path.join(root, "output", "field_avg", name)
        sums = np.concatenate([want[nm].ravel() for nm in abi.AVG_NAMES])
        wpath = os.path.join(root, name + ".want")
        fileio.write_fav(wpath, c.settings["re"], f["n"], sums, f["timeinit"], f["timeend"],
                         int(f["ihistinit"]), int(f["ihistend"]), 1)
        with open(fpath, "rb") as a, open(wpath, "rb") as b:
            assert a.read() == b.read(), name
    comb = fileio.read_fav(os.path.join(root, "output", "field_avg", "combined", "fav0000001-0000006"), 1)
    assert np.array_equal(comb["ssavg"], avgs[0]["ssavg"] + avgs[1]["ssavg"])
    assert comb["timeinit"] == 0.0 and comb["timeend"] == reps[-1]["time"]
    sol.close()


@pytest.mark.parametrize("name", ["cylinder_array", "cylinder_zft_mixed"])
def test_exec_ib_cases(tmp_path, name):
    if name == "cylinder_array":
        c = cases.cylinder_array(48, 40, 8)
    else:
        c = cases.cylinder(64, 48, 8, precision=abi.PREC_MIXED)
    root = str(tmp_path)
    sdir = fileio.write_case_dir(root, c, nend=4, nprint=10, npin=2)
    run_exec(sdir)
    s = dict(c.settings); s.update(iread=1, ireset=0, nend=4, nprint=10, npin=2)
    rc = restart_case(root, c, s)
    sol = leswht_gb300.gpu_solver(rc)
    reps = [sol.step() for _ in range(4)]
    # NEND is not a multiple of NPRINT: the final writefield of solver.f90:190
    check_field(os.path.join(root, "output", "field", "fld0000002"), rc, sol.fields(), reps[-1], s["ihtrans"])
    hist = lines(os.path.join(root, "output", "ftr", "fhist.dat"))
    assert hist == [FMT5 % (r["time"], r["dt"], r["cflmax"], r["dvmax"], r["qmmax"]) for r in reps[1::2]]
    if s["ibmon"] == 1:
        cd = lines(os.path.join(root, "output", "ftr", "fcdcl.dat"))
        assert [ln[:58] for ln in cd] == [(FMT7 % (r["time"], *r["cd"], 0, 0, 0))[:58] for r in reps[1::2]]
    if s["ihtrans"] == 1:
        hf = lines(os.path.join(root, "output", "ftr", "fheatflux.dat"))
        assert [ln[:58] for ln in hf] == [(FMT7 % (r["time"], *r["heat_flux"], 0, 0, 0))[:58] for r in reps[1::2]]
    sol.close()
