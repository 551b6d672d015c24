"""Generate the golden fixtures in this folder from the reference's own code.

Runs the reference's kernels and set-up lines compiled for the host
(oracle/_ref/libpoe2d_ref.so, built by oracle/build_ref.sh from the reference
sources) and stores inputs and outputs as small .npz files:

  ref_setup.npz  medium-ID model -> the 8 coefficient planes with the
                 reference's own fluid table (cu:553-575, 646-661, 682-713),
                 and the C-PML profiles (cu:840-845, 985-1159)
  ref_loop.npz   NSTEP steps of the six-launch loop (cu:1628-1634) on a
                 heterogeneous 41 x 33 grid: final 12 fields and the save1
                 recordings (cu:114-201)

Usage: python tests/golden/make_golden.py   (needs the reference tree)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle import oracle as O  # noqa: E402

# a stable poroelastic table for the loop (IDs 0..3): K_f, eta, kappa, phi, a, rho_f
LOOP_TABLE = np.array([[2.25e09, 1e-3, 1e-12, 0.2, 2.0, 1000.0],
                       [2.25e09, 1e-3, 5e-13, 0.25, 2.2, 1000.0],
                       [0.7e09, 0.03, 5e-13, 0.25, 2.0, 700.0],
                       [0.02e09, 1.0e-5, 5e-13, 0.25, 2.0, 100.0]], np.float32)


def model(NX, NZ, seed):
    rng = np.random.default_rng(seed)
    sh = (NZ + 1, NX + 1)
    medium = rng.integers(0, 4, size=sh).astype(np.float32)
    cp = rng.uniform(2500, 3200, size=sh).astype(np.float32)
    cs = rng.uniform(1200, 1600, size=sh).astype(np.float32)
    rho = rng.uniform(2000, 2600, size=sh).astype(np.float32)
    return medium, cp, cs, rho


def main():
    if not O.ref_available():
        sys.exit("reference harness not built (sh oracle/build_ref.sh)")
    NX, NZ, dx, dt, f0, npml = 40, 32, 1.25, 95e-6, 200.0, 8
    medium, cp, cs, rho = model(NX, NZ, 7)
    coef_ref = O.ref_coeffs(medium, cp, cs, rho)
    px, pz, rc = O.ref_pml(NX, NZ, dx, dx, dt, npml, f0, float(cp.max()))
    np.savez_compressed(os.path.join(HERE, "ref_setup.npz"), NX=NX, NZ=NZ, dx=dx, dt=dt, f0=f0, npml=npml,
                        medium=medium, cp=cp, cs=cs, rho=rho, coef=coef_ref, prof_x=px, prof_z=pz)
    # loop: stable coefficients from the oracle restatement (checked equal to the
    # reference lines with the reference table above), profiles from the reference
    coef_loop, bad = O.coeffs_from_medium(medium, cp, cs, rho, LOOP_TABLE)
    assert bad == 0
    nsteps, isrc, jsrc, panj, panj2, a0, a1 = 160, 20, 16, 4, 5, 12, 20
    fields, seis, ig = O.ref_run(NX, NZ, dx, dt, isrc, jsrc, f0, coef_loop, px, pz, nsteps, panj, panj2, a0, a1)
    keep = {k: fields[k] for k in O.FIELDS[:12]}
    np.savez_compressed(os.path.join(HERE, "ref_loop.npz"), NX=NX, NZ=NZ, dx=dx, dt=dt, f0=f0, npml=npml,
                        nsteps=nsteps, isrc=isrc, jsrc=jsrc, panj=panj, panj2=panj2, a0=a0, a1=a1, i_gpu=ig,
                        coef=coef_loop, prof_x=px, prof_z=pz, **keep, **seis)
    print("wrote ref_setup.npz, ref_loop.npz; i_gpu =", ig)


if __name__ == "__main__":
    main()
