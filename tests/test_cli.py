"""The drop-in driver poe2d_run: the reference program's inputs and outputs.

CPU tests use --dry-run (inputs read and checked, coefficients and C-PML
profiles built, mediumrho.ctxt written, no GPU).  The GPU test runs a small
model end to end and checks every output file, byte for byte, against the
same run through the library (traces, snapshots) formatted the way the
reference's std::ofstream prints floats (cu:1772-1905).
"""
import os
import subprocess

import numpy as np
import pytest

from poe2d_gb300 import build as B

NX, NZ = 119, 99


def _cli():
    B.build()
    assert os.path.exists(B.CLI)
    return B.CLI


def _write_case(d, order="x", nstep=130, isrc=60, jsrc=50, f0=200.0, ids=None):
    from poe2d_gb300.patchy import write_bin
    rng = np.random.default_rng(5)
    sh = (NZ + 1, NX + 1)
    medium = (ids if ids is not None else rng.integers(0, 4, size=sh)).astype(np.float32)
    cp = rng.uniform(2600, 3300, size=sh).astype(np.float32)
    cs = rng.uniform(1300, 1700, size=sh).astype(np.float32)
    rho = rng.uniform(2100, 2500, size=sh).astype(np.float32)
    for name, a in (("m.bin", medium), ("cp.bin", cp), ("cs.bin", cs), ("rho.bin", rho)):
        write_bin(os.path.join(d, name), a, order=order)
    with open(os.path.join(d, "input1.txt"), "w") as f:
        f.write("%d\n%d %d\n%d\n%d\n" % (nstep, isrc, jsrc, 30, 70))
    with open(os.path.join(d, "input2.txt"), "w") as f:
        f.write("%g\n" % f0)
    # stable poroelastic fluids (the reference's own table is its elastic limit, phi = 1e-6)
    from tests.golden.make_golden import LOOP_TABLE
    np.savetxt(os.path.join(d, "fluid.txt"), np.asarray(LOOP_TABLE, np.float64), fmt="%.9g")
    return medium, cp, cs, rho


def _args(d, order="x", extra=()):
    return [_cli(), "--nx", str(NX), "--nz", str(NZ), "--dx", "0.5", "--dt", "5e-5", "--panj", "10", "--panj2",
            "12", "--samp", "64", "--npml", "10", "--medium", "m.bin", "--cp", "cp.bin", "--cs", "cs.bin", "--rho",
            "rho.bin", "--order", order, "--fluid", os.path.join(d, "fluid.txt"), "--in", d, "--out", d] + list(extra)


def test_missing_inputs_message(tmp_path):
    r = subprocess.run([_cli(), "--in", str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 1 and "File not opened..." in r.stdout


@pytest.mark.parametrize("order", ["x", "z"])
def test_dry_run_reads_both_orders(tmp_path, order):
    d = str(tmp_path)
    medium, cp, cs, rho = _write_case(d, order)
    r = subprocess.run(_args(d, order, ["--dry-run"]), capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "grid 120 x 100" in r.stdout
    dump = np.fromfile(os.path.join(d, "mediumrho.ctxt"), "<f4").reshape(NZ + 1, NX + 1)
    assert np.array_equal(dump, cp)          # cu:1476-1487 writes cp, x fastest


def test_bad_medium_id_and_short_file(tmp_path):
    d = str(tmp_path)
    ids = np.zeros((NZ + 1, NX + 1))
    ids[3, 4] = 7                             # no fluid row 7
    _write_case(d, ids=ids)
    r = subprocess.run(_args(d, extra=["--dry-run"]), capture_output=True, text=True)
    assert r.returncode == 1 and "medium" in r.stderr
    _write_case(d)
    with open(os.path.join(d, "cs.bin"), "r+b") as f:
        f.truncate(100)
    r = subprocess.run(_args(d, extra=["--dry-run"]), capture_output=True, text=True)
    assert r.returncode == 1 and "expected" in r.stderr


def test_argument_and_input_errors_exit_with_a_message(tmp_path):
    """Errors the reference would crash on or ignore are reported: a fluid table
    that is not rows of 6 values or is missing, unknown options or missing
    values (exit 2), a bad --order, a source outside the grid."""
    d = str(tmp_path)
    _write_case(d)
    with open(os.path.join(d, "fluid.txt"), "a") as f:
        f.write("1.0\n")                                     # 4 x 6 + 1 values
    r = subprocess.run(_args(d, extra=["--dry-run"]), capture_output=True, text=True)
    assert r.returncode == 1 and "rows of 6 values" in r.stderr
    args = _args(d, extra=["--dry-run"])
    args[args.index("--fluid") + 1] = os.path.join(d, "no_such_table.txt")
    r = subprocess.run(args, capture_output=True, text=True)
    assert r.returncode == 1 and "cannot open" in r.stderr
    r = subprocess.run([_cli(), "--frobnicate"], capture_output=True, text=True)
    assert r.returncode == 2 and "unknown option" in r.stderr
    r = subprocess.run([_cli(), "--nx"], capture_output=True, text=True)
    assert r.returncode == 2 and "missing value" in r.stderr
    r = subprocess.run([_cli(), "--order", "y"], capture_output=True, text=True)
    assert r.returncode == 2
    _write_case(d, isrc=NX + 5)                             # fresh, valid table; source off the grid
    r = subprocess.run(_args(d, extra=["--dry-run"]), capture_output=True, text=True)
    assert r.returncode == 1 and "outside the grid" in r.stderr


def test_courant_failure_returns_like_the_reference(tmp_path):
    d = str(tmp_path)
    _write_case(d)
    args = _args(d, extra=["--dry-run"])
    args[args.index("--dt") + 1] = "5e-4"
    r = subprocess.run(args, capture_output=True, text=True)
    assert r.returncode == 0 and "time step is too large" in r.stdout


def test_ref_steps_runs_the_references_whole_chunks(tmp_path):
    """The reference's loop runs NSTEP/samp*samp steps (cu:1620); --ref-steps
    does the same, without it every step runs."""
    d = str(tmp_path)
    _write_case(d, nstep=130)
    r = subprocess.run(_args(d, extra=["--dry-run"]), capture_output=True, text=True)
    assert r.returncode == 0 and "130 steps run" in r.stdout, r.stdout
    r = subprocess.run(_args(d, extra=["--dry-run", "--ref-steps"]), capture_output=True, text=True)
    assert r.returncode == 0 and "NSTEP=130" in r.stdout and "128 steps run" in r.stdout, r.stdout
    _write_case(d, nstep=50)                                  # NSTEP < samp: the reference runs no step
    r = subprocess.run(_args(d, extra=["--dry-run", "--ref-steps"]), capture_output=True, text=True)
    assert r.returncode == 0 and " 0 steps run" in r.stdout, r.stdout


def _fmt_rows(a):
    return "".join("".join("%g " % float(v) for v in row) + "\n" for row in a)


@pytest.mark.gpu
def test_cli_outputs_match_library_run(tmp_path, poe):
    d = str(tmp_path)
    nstep, isrc, jsrc, f0 = 130, 60, 50, 200.0
    medium, cp, cs, rho = _write_case(d, "z", nstep, isrc, jsrc, f0)
    r = subprocess.run(_args(d, "z"), capture_output=True, text=True)
    assert r.returncode == 0, r.stderr

    from tests.golden.make_golden import LOOP_TABLE
    g = poe.grid(NX, NZ, 0.5, 5e-5)
    coef = poe.coeffs_from_medium(g, medium, cp, cs, rho, LOOP_TABLE)
    px, pz = poe.pml_profiles(g, 10, f0, float(cp.max()))
    rec = poe.ref_receivers(g, isrc, jsrc, 10, 12, 30, 70)
    with poe.Solver(g, coef, px, pz) as s:
        s.add_shot(poe.source(isrc, jsrc, poe.SRC_REF_DGAUSS_P, f0, 1.0, 0.4), rec)
        snaps = {}
        for k in (64, 128):
            s.run(k - s.steps())
            snaps[k] = (s.field("vz"), s.field("vx"))
        s.run(nstep - s.steps())
        tr = s.traces()
    for k, (vz, vx) in snaps.items():
        assert np.array_equal(np.fromfile(os.path.join(d, "vz%05d.vzo" % k), "<f4").reshape(vz.shape), vz)
        assert np.array_equal(np.fromfile(os.path.join(d, "vx%05d.vxo" % k), "<f4").reshape(vx.shape), vx)
    assert not os.path.exists(os.path.join(d, "vz%05d.vzo" % 130))
    cols = {"recvspvz%08d.vsp": tr[:, 0:10], "recvspvx%08d.vsp": tr[:, 10:20], "rechorvz%08d.hor": tr[:, 20:32],
            "rechorvx%08d.hor": tr[:, 32:44]}
    for pat, a in cols.items():
        with open(os.path.join(d, pat % int(f0))) as f:
            assert f.read() == _fmt_rows(a), pat
    for i, pat in enumerate(("recats%08d.ats", "recbwh%08d.bwh", "recsrc%08d.src")):
        with open(os.path.join(d, pat % int(f0))) as f:
            assert f.read() == "".join("%g " % float(v) for v in tr[:, 45 + i]), pat


@pytest.mark.gpu
def test_cli_restart_from_checkpoint_gives_the_same_files(tmp_path):
    a, b = tmp_path / "a", tmp_path / "b"
    a.mkdir()
    b.mkdir()
    _write_case(str(a), nstep=150)
    _write_case(str(b), nstep=150)
    ck = str(tmp_path / "ck.img")
    r = subprocess.run(_args(str(a), extra=["--checkpoint", ck]), capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert os.path.getsize(ck) > 0                  # image of step 128
    r = subprocess.run(_args(str(b), extra=["--restart", ck]), capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    for name in ("recvspvz00000200.vsp", "rechorvx00000200.hor", "recsrc00000200.src"):
        assert (a / name).read_bytes() == (b / name).read_bytes(), name
    assert not (b / "vz00064.vzo").exists()          # restarted past the first snapshot


@pytest.mark.gpu
def test_cli_ref_steps_writes_zero_rows_past_the_last_chunk(tmp_path, poe):
    """With --ref-steps and NSTEP % samp != 0 the files hold NSTEP rows: the
    first NSTEP/samp*samp are the run's, the rest are 0, as the reference
    writes its cleared trace arrays (cu:1251-1305, 1737-1905)."""
    d = str(tmp_path)
    nstep, isrc, jsrc, f0 = 130, 60, 50, 200.0
    medium, cp, cs, rho = _write_case(d, "x", nstep, isrc, jsrc, f0)
    r = subprocess.run(_args(d, "x", ["--ref-steps", "--no-snapshots"]), capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    from tests.golden.make_golden import LOOP_TABLE
    g = poe.grid(NX, NZ, 0.5, 5e-5)
    coef = poe.coeffs_from_medium(g, medium, cp, cs, rho, LOOP_TABLE)
    px, pz = poe.pml_profiles(g, 10, f0, float(cp.max()))
    rec = poe.ref_receivers(g, isrc, jsrc, 10, 12, 30, 70)
    with poe.Solver(g, coef, px, pz) as s:
        s.add_shot(poe.source(isrc, jsrc, poe.SRC_REF_DGAUSS_P, f0, 1.0, 0.4), rec)
        s.run(128)
        tr = np.zeros((nstep, len(rec)), np.float32)
        tr[:128] = s.traces()
    assert np.abs(tr[:128]).max() > 0
    with open(os.path.join(d, "rechorvz%08d.hor" % int(f0))) as f:
        assert f.read() == _fmt_rows(tr[:, 20:32])
    with open(os.path.join(d, "recsrc%08d.src" % int(f0))) as f:
        assert f.read() == "".join("%g " % float(v) for v in tr[:, 47])
    assert not os.path.exists(os.path.join(d, "vz%05d.vzo" % 128))
