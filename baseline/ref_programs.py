"""Times the reference's own programs, staged by baseline/stage_ref.sh into
baseline/_ref/src/, on the machine that runs this (the benchmark's GPU machine).

* The CUDA program (seismic_CPML_2D_poroelastic_withCUDA.cu) runs its own
  six-launch loop (cu:1596-1636) and prints, per chunk of samp steps, the
  cumulative time of its kernels measured with its own CUDA events (cu:1601,
  1624, 1637-1648, "Waktu perhitungan"); that figure is the loop time.  Its
  launch geometry needs (NX+1) % 10 == 0 (cu:1597-1600), so a 2001 x 2001
  benchmark grid runs padded to 2010 x 2010 and cell-updates are counted on
  the padded grid.
* The serial C++ twin (seismic_CPML_2d_poroelastic.cpp) runs chunks of samp+1
  steps (cpp:614-616) and writes a vz snapshot after each (cpp:840-855); its
  own timer is broken (t2 = clock_t(), cpp:920-926), so the step time is read
  off the snapshot files' modification times: the gap between the first two
  snapshots is one chunk of samp+1 steps plus one chunk's output.  Its
  out-of-bounds trace writes (sseismo0[i_steps-1] with i_steps = 0 and rows
  past NSTEP, cpp:585-592, 678, 720) corrupt its heap, and it aborts after a
  few chunks; the first two snapshots are written before that.

Both read the reference's input files: input1.txt (NSTEP ISOURCE JSOURCE
a0_pos a1_pos), input2.txt (f0) and four float32 grids named as the
reference names them (cu:606-644), written here from the benchmark's patchy
model: medium IDs 1 (water-bearing row of the reference's fluid table,
cu:565-575) and 3 (gas row), cp 3411 m/s, cs 1857 m/s, rho 2320 kg/m3.
"""
from __future__ import annotations

import os
import re
import shutil
import subprocess
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "_ref", "src")
BUILD = os.path.join(HERE, "_ref", "build")


def staged():
    return os.path.exists(os.path.join(SRC, "ref_cuda.cu")) and os.path.exists(os.path.join(SRC, "ref_cpu.cpp"))


def _defines(n, dx, dt, panj, samp, npml):
    return {"POE_NX": n - 1, "POE_NZ": n - 1, "POE_DX": "%rf" % dx, "POE_DT": "%rf" % dt, "POE_PANJ": panj,
            "POE_PANJ2": panj, "POE_SAMP": samp, "POE_NPML": npml}


def build(kind, defs):
    """Compile the staged program kind ("cuda" or "cpu") with the given
    constants (cached per set of constants); returns the executable."""
    os.makedirs(BUILD, exist_ok=True)
    tag = "_".join("%s" % v for v in defs.values()).replace(".", "p").replace("-", "m")
    exe = os.path.join(BUILD, "ref_%s_%s" % (kind, tag))
    if os.path.exists(exe):
        return exe
    d = ["-D%s=%s" % kv for kv in defs.items()]
    if kind == "cuda":
        nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
        cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-w", "-I", SRC] + d + [
            os.path.join(SRC, "ref_cuda.cu"), "-o", exe]
    else:
        cmd = [shutil.which("g++") or "g++", "-O3", "-w", "-I", SRC, "-include", "win.h"] + d + [
            os.path.join(SRC, "ref_cpu.cpp"), "-o", exe]
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("building the reference's %s program failed: %s" % (kind, (out.stderr or out.stdout)[-400:]))
    return exe


def write_inputs(d, ids, nstep, isrc, jsrc, a0, a1, f0):
    """The reference's input files for a model of medium ids (0 background,
    1 gas), x fastest as the reference reads them (cu:606-644, 685)."""
    n1, n0 = ids.shape
    medium = np.where(ids > 0, 3.0, 1.0).astype("<f4")
    for name, a in (("poro", medium), ("cp", np.full(ids.shape, 3411.0)), ("cs", np.full(ids.shape, 1857.0)),
                    ("rho", np.full(ids.shape, 2320.0))):
        np.ascontiguousarray(a, "<f4").tofile(os.path.join(d, "mar_%s_2440x13600.bin" % name))
    with open(os.path.join(d, "input1.txt"), "w") as f:
        f.write("%d\n%d %d\n%d\n%d\n" % (nstep, isrc, jsrc, a0, a1))
    with open(os.path.join(d, "input2.txt"), "w") as f:
        f.write("%g\n" % f0)


def time_cuda(ids, dx, dt, npml, f0, nstep=2000, samp=1000, timeout=600):
    """The reference's CUDA loop on this GPU: {value (Gcell-updates/s), ...}."""
    n = ids.shape[0]
    defs = _defines(n, dx, dt, n // 10, samp, npml)
    exe = build("cuda", defs)
    with tempfile.TemporaryDirectory(prefix="poe2d_ref_") as d:
        write_inputs(d, ids, nstep, n // 2, npml, 100, 200, f0)
        t0 = time.perf_counter()
        out = subprocess.run([exe], cwd=d, capture_output=True, text=True, timeout=timeout, stdin=subprocess.DEVNULL)
        wall = time.perf_counter() - t0
    secs = [float(v) for v in re.findall(r"Waktu perhitungan\s*=\s*([0-9.]+)\s*s", out.stdout)]
    if out.returncode != 0 or len(secs) != nstep // samp or secs[-1] <= 0:
        raise RuntimeError("the reference's CUDA program did not finish its loop (rc %d): %s"
                           % (out.returncode, (out.stdout + out.stderr)[-300:]))
    return {"value": n * n * nstep / secs[-1] / 1e9, "unit": "Gcell-updates/s", "grid": [n, n], "steps": nstep,
            "loop_s": secs[-1], "process_wall_s": wall,
            "how": "its own CUDA-event time of the %d-step loop (cu:1601-1648), %d x %d cells (padded for its "
                   "10 x 10 launch geometry)" % (nstep, n, n)}


def time_cpu(ids, dx, dt, npml, f0, samp=10, timeout=900):
    """The reference's serial C++ loop on one host core: {value, ...} from the
    gap between its first two vz snapshots (samp+1 steps and one chunk's output)."""
    n = ids.shape[0]
    defs = _defines(n, dx, dt, n // 10, samp, npml)
    exe = build("cpu", defs)
    with tempfile.TemporaryDirectory(prefix="poe2d_refcpu_") as d:
        write_inputs(d, ids, 3 * samp, n // 2, npml, 100, 200, f0)
        t0 = time.perf_counter()
        out = subprocess.run([exe], cwd=d, capture_output=True, text=True, timeout=timeout, stdin=subprocess.DEVNULL)
        wall = time.perf_counter() - t0
        snaps = [os.path.join(d, "vz%05d.vzo" % (k * samp)) for k in (1, 2)]
        if not all(os.path.exists(p) for p in snaps):
            raise RuntimeError("the reference's CPU program wrote no two snapshots (rc %d): %s"
                               % (out.returncode, (out.stdout + out.stderr)[-300:]))
        gap = os.stat(snaps[1]).st_mtime_ns - os.stat(snaps[0]).st_mtime_ns
    secs = gap * 1e-9
    return {"value": n * n * (samp + 1) / secs / 1e9, "unit": "Gcell-updates/s", "cores": 1, "grid": [n, n],
            "sample": "%d steps between its first two vz snapshots, %.1f s (its own timer is broken, cpp:920-926; "
                      "the program then aborts on its out-of-bounds trace writes, rc %d)" % (samp + 1, secs,
                                                                                            out.returncode),
            "process_wall_s": wall}
