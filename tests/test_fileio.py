"""The reference's on-disk formats (Fortran records of writefield / prefld /
field_avg, the text inputs of readsettings / readbcs / readgeom and the
pre-processor tables) and the compiled driver's readers of them, checked on
the CPU: lesgpu_exec --dry-run parses a case directory and prints what it
read, which must be exactly the case that wrote it."""
import subprocess

import numpy as np
import pytest

import leswht_gb300
from leswht_gb300 import abi, cases, fileio


def seqsum(a):
    """The plain left-to-right sum (the order the driver adds in)."""
    a = np.asarray(a, dtype=np.float64).ravel()
    return float(np.cumsum(a)[-1]) if a.size else 0.0


def test_records_round_trip(tmp_path):
    recs = [b"", b"abc", np.arange(5, dtype="<f8").tobytes()]
    p = tmp_path / "r.bin"
    fileio.write_records(str(p), recs)
    raw = p.read_bytes()
    assert raw[:4] == b"\x00\x00\x00\x00" and raw[4:8] == b"\x00\x00\x00\x00"
    assert raw[8:12] == (3).to_bytes(4, "little")
    assert fileio.read_records(str(p)) == recs


def test_field_round_trip(tmp_path):
    c = cases.channel(16, 16, 8)
    p = str(tmp_path / "fld0000007")
    fileio.write_field(p, c.settings, c.grid, c.fields, ihist=7, m=70, time=1.25, dt=0.002)
    r = fileio.read_field(p, c.grid, ihtrans=1, tsol_i=c.settings["tsol_i"])
    assert (r["ihist"], r["m"], r["time"], r["dt"]) == (7, 70, 1.25, 0.002)
    g = c.grid
    n1, n2, n3 = g.n1, g.n2, g.n3
    sl = {"u": np.s_[0:n3 + 1, 0:n2 + 1, 1:n1 + 1], "v": np.s_[0:n3 + 1, 1:n2 + 1, 0:n1 + 1],
          "w": np.s_[1:n3 + 1, 0:n2 + 1, 0:n1 + 1], "p": np.s_[1:n3, 1:n2, 1:n1], "t": np.s_[1:n3, 1:n2, 1:n1]}
    for k, s in sl.items():
        assert np.array_equal(r[k][s], c.fields[k][s]), k
    recs = fileio.read_records(p)
    assert len(recs) == 10 and len(recs[5]) == 8 * n1 * (n2 + 1) * (n3 + 1)


def test_fav_reader(tmp_path):
    n = (3, 2, 2)
    vals = [np.full(n[::-1], float(q)) for q in range(23)]
    recs = [np.array(n, "<i8").tobytes() + np.array([150.0], "<f8").tobytes(),
            np.array([1.0, 2.0, 10.0, 20.0], "<f8").tobytes()]
    groups = [1, 1, 1, 6, 1, 1, 3, 6, 1, 1, 1]
    q = 0
    for gsz in groups:
        recs.append(b"".join(vals[q + e].tobytes() for e in range(gsz)))
        q += gsz
    p = str(tmp_path / "fav0000010-0000020")
    fileio.write_records(p, recs)
    f = fileio.read_fav(p, ihtrans=1)
    assert f["n"] == n and f["ihistend"] == 20.0 and f["timeinit"] == 1.0
    assert f["uiujavg"].shape == (6, 2, 2, 3) and f["uiujavg"][5, 0, 0, 0] == 8.0
    assert f["t2avg"][0, 0, 0] == 22.0


def _dry_run(sdir):
    exe = leswht_gb300.exec_path()
    out = subprocess.run([str(exe), "--dry-run"], cwd=sdir, capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    d = {}
    for line in out.stdout.splitlines():
        k, *v = line.split()
        d[k] = v
    return d


CASES = {
    "channel": lambda: cases.channel(16, 16, 8),
    "cylinder_array": lambda: cases.cylinder_array(48, 40, 8),
    "cylinder_zft": lambda: cases.cylinder(64, 48, 8, precision=abi.PREC_MIXED),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_exec_reads_case_dir(tmp_path, name):
    c = CASES[name]()
    sdir = fileio.write_case_dir(str(tmp_path), c, nend=5, nprint=2, npin=1)
    d = _dry_run(sdir)
    s = dict(c.settings)
    s.update(iread=1, ireset=0, nend=5, nprint=2, npin=1)
    for k, v in s.items():
        if k == "body":
            for bk, bv in v.items():
                got = d["body." + bk][0]
                assert (int(got) if bk == "kind" else float(got)) == bv, bk
            continue
        if k not in d:
            continue
        got = d[k][0]
        assert (int(got) if isinstance(v, (int, np.integer)) else float(got)) == v, k
    for key in ("re", "pr", "bc_ybtm", "xprdic", "poisson", "precision", "ibmon", "ihtrans"):
        assert key in d
    g = c.grid
    assert [int(x) for x in d["grid"]] == [g.n1, g.n2, g.n3, g.n1m, g.n2m, g.n3m]
    assert float(d["ymp"][1]) == seqsum(g.ymp) and float(d["c2cy"][1]) == seqsum(g.c2cy)
    t = c.ibm
    for l in range(4):
        row = d[f"ibm{l}"]
        if s["ibmon"] != 1 or (l == 3 and s["ihtrans"] != 1):
            assert int(row[0]) == 0 and int(row[1]) == 0
            continue
        assert int(row[0]) == t["nintp"][l] and int(row[1]) == t["nbody"][l]
        assert int(row[2]) == int(np.sum(t["fc"][l])) and int(row[3]) == int(np.sum(t["intpindx"][l]))
        assert float(row[4]) == seqsum(t["geomfac"][l])
    if s["ibmon"] == 1 and s["iles"] == 1:
        assert [int(x) for x in d["nzero"]] == [t["nzero"], int(np.sum(t["inz"])), int(np.sum(t["jnz"])),
                                                int(np.sum(t["knz"]))]
        assert int(d["nwall"][1]) == int(np.sum(t["nwall_dvm"]))
    assert [float(x) for x in d["state"]] == [c.ihist, c.m, c.time, c.dt]
    # prefld's ghost copies are not idempotent at the corner ghosts (the z
    # copy of u skips i = 0, so u(0, j, 0) comes from before or after it), so
    # the state after a read is prefld applied to the stored records
    r = fileio.read_field(sdir + "/../output/field/fld0000000", g, s["ihtrans"], s["tsol_i"])
    U, V, W, P, T = cases.prefld_apply(s, g, r["u"], r["v"], r["w"], r["p"], r["t"])
    if s["ihtrans"] != 1:
        T = np.full(g.shape, s["tsol_i"])
    got = [float(x) for x in d["fields"]]
    assert got == [seqsum(a) for a in (U, V, W, P, T)]


def test_exec_rejects_mismatched_field(tmp_path):
    c = cases.channel(16, 16, 8)
    sdir = fileio.write_case_dir(str(tmp_path), c, nend=1)
    small = cases.channel(8, 16, 8)
    fileio.write_field(str(tmp_path / "output" / "field" / "fld0000000"), small.settings, small.grid, small.fields,
                       0, 0, 0.0, 0.002)
    exe = leswht_gb300.exec_path()
    out = subprocess.run([str(exe), "--dry-run"], cwd=sdir, capture_output=True, text=True, timeout=120)
    assert out.returncode != 0 and "DOES NOT MATCH" in out.stderr
