"""Generate the golden fixtures in this directory from the reference's OWN
sources (compiled here by `make -C oracle ref`, see oracle/Makefile).

Each fixture holds the seeded input state, the deck parameters and the state
the reference produced after the given number of RK4 steps.  Run from the
repository root:

    python tests/golden/make_golden.py [case ...]

The reference has no golden vectors or tests of its own, so these fixtures
are the pin for the oracle (tests/test_oracle_pin.py) and for the GPU path
(tests/test_gpu_parity.py), which must not need the reference at run time.
"""
import dataclasses
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "triplyperiodic-modified_gb300"))

import pyoracle as po  # noqa: E402
from tpm import inputs, params as P  # noqa: E402

CASES = {
    # heated two-way coupled box, power-of-two grid, fixed Poisson iteration count
    "heated16_2steps": dict(N=16, npart=1000, nu=0.02, A=0.1, tau_p=0.1, mass_loading=0.5,
                            heating_Q=0.5, iterations=3, epsilon=0.0, seed=11, nsteps=2),
    # non-power-of-two grid (radix 3), gravity on gas and particles, cooling
    # branch, and the threshold switch of params.cpp:80-86 after the first step
    "cooled24_gravity_switch": dict(N=24, npart=500, nu=0.01, A=0.05, tau_p=0.2,
                                    mass_loading=0.3, heating_Q=0.2, iterations=20,
                                    epsilon=1e-13, seed=12, nsteps=2,
                                    extra=dict(cooling=1, ParticleGravity=1, gz1=-0.5,
                                               gz2=-1.0, A2=0.2, threshold=0.001)),
    # the loop as shipped (particle stage disabled, simulation.cpp:64)
    "shipped24_1step": dict(N=24, npart=100, nu=0.02, A=0.1, tau_p=0.1, mass_loading=0.2,
                            heating_Q=0.0, iterations=2, epsilon=0.0, seed=13, nsteps=1,
                            as_shipped=True),
    # passive scalar transport (grid.cpp:743-772) with each source type
    "scalar16_source_2steps": dict(N=16, npart=1000, nu=0.02, A=0.1, tau_p=0.1,
                                   mass_loading=0.5, heating_Q=0.5, iterations=20,
                                   epsilon=1e-13, seed=31, nsteps=2, scalar=True,
                                   extra=dict(solve_for_scalar=1, D_M=0.03, S1_type=0)),
    "scalar24_meangrad_2steps": dict(N=24, npart=800, nu=0.01, A=0.1, tau_p=0.2,
                                     mass_loading=0.3, heating_Q=0.0, iterations=20,
                                     epsilon=1e-13, seed=32, nsteps=2, scalar=True,
                                     extra=dict(solve_for_scalar=1, D_M=0.01, S1_type=1)),
    # grid::Statistics after each of 3 steps, as the reference writes it
    # (<name>.dat files, 6 significant digits)
    "stats16_3steps": dict(N=16, npart=2000, nu=0.02, A=0.1, tau_p=0.1, mass_loading=0.5,
                           heating_Q=0.5, iterations=20, epsilon=1e-13, seed=21, nsteps=3,
                           stats=True),
}


def make(name, c):
    p = P.physical(c["N"], c["npart"], nu=c["nu"], A=c["A"], tau_p=c["tau_p"],
                   mass_loading=c["mass_loading"], heating_Q=c["heating_Q"],
                   iterations=c["iterations"], epsilon=c["epsilon"])
    s = inputs.make_state(p, c["npart"], seed=c["seed"])
    p = p.replace(dt=inputs.cfl_dt(p, s.RU), **c.get("extra", {}))
    if c.get("scalar"):
        s.PS = inputs.passive_scalar(p, c["seed"])
    ref = po.run_reference(p, s, c["nsteps"], as_shipped=c.get("as_shipped", False),
                           stats=c.get("stats", False))
    out = dict(
        params=json.dumps(dataclasses.asdict(p)), nsteps=c["nsteps"],
        as_shipped=int(c.get("as_shipped", False)),
        in_RU=s.RU, in_Rho=s.Rho, in_P=s.P, in_P0=s.P0,
        **{f"in_part_{q}": s.part[q] for q in list(inputs.PQ) + ["flag"]},
        RU=ref["RU"], RU_int=ref["RU_int"], Rho=ref["Rho"], P=ref["P"], C=ref["C"],
        Q=ref["RHS_Part_Temp"], P0=ref["P0"], T_cur=ref["T_cur"],
        **{f"part_{q}": ref["part"][q] for q in list(inputs.PQ) + ["flag", "RHS_T"]},
        **{f"stat_{k}": v for k, v in ref.get("stats", {}).items()},
        **({"in_PS": s.PS, "PS": ref["Passive_Scalar"]} if c.get("scalar") else {}),
    )
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(name, "written")


if __name__ == "__main__":
    if not po.have_reference():
        po.build()
    names = sys.argv[1:] or list(CASES)
    for name in names:
        make(name, CASES[name])
