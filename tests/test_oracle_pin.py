"""Pin the C oracle (oracle/tpm_oracle.c) to the reference.

1. Against the committed golden fixtures, which the reference's own sources
   produced (tests/golden/make_golden.py): <= 1e-12 relative per field, and
   bit-identical on the loop as shipped (no particle stage), where summation
   order cannot differ.
2. Where the reference build exists (this container), against fresh runs on
   new seeds.
"""
import numpy as np
import pytest

from conftest import rel_err
from golden import NAMES, SCALAR_NAMES, load
from tpm import inputs, params as P

TOL = 1e-12  # relative, per field (FP64 parity bar)


def run_oracle(oracle_lib, p, s, nsteps, with_particles=True):
    o = oracle_lib.Oracle(p, s.npart)
    o.load(s)
    o.initialize()
    for _ in range(nsteps):
        o.step(with_particles)
    return o


def compare(o, ref, tol, bitwise=False):
    got = {"RU": o.get_field("RU"), "RU_int": o.get_field("RU_INT"), "Rho": o.get_field("RHO"),
           "P": o.get_field("P")}
    for k, v in got.items():
        if bitwise:
            assert np.array_equal(v, ref[k]), k
        else:
            assert rel_err(v, ref[k]) <= tol, (k, rel_err(v, ref[k]))
    part = o.get_particles(0)
    assert np.array_equal(part["flag"], ref["part"]["flag"])
    for q in inputs.PQ:
        if bitwise:
            assert np.array_equal(part[q], ref["part"][q]), q
        else:
            assert rel_err(part[q], ref["part"][q]) <= tol, (q, rel_err(part[q], ref["part"][q]))
    return got


@pytest.mark.parametrize("name", NAMES)
def test_oracle_matches_golden(oracle_lib, name):
    p, s, ref, nsteps, as_shipped = load(name)
    o = run_oracle(oracle_lib, p, s, nsteps, with_particles=not as_shipped)
    compare(o, ref, TOL, bitwise=as_shipped)
    if not as_shipped:
        assert rel_err(o.get_field("C"), ref["C"]) <= TOL
        # the heat exchange is a difference of nearly equal temperatures, so its
        # relative roundoff is amplified; still far inside the FP64 bar
        assert rel_err(o.get_field("Q"), ref["Q"]) <= 1e-11
        assert rel_err(o.get_rhs_t(), ref["part"]["RHS_T"]) <= 1e-11
    sc = o.scalars()
    assert abs(sc["P0"] - ref["P0"]) <= 1e-14 * abs(ref["P0"])
    assert sc["T_cur"] == ref["T_cur"]


def test_oracle_cell_indices_match_golden(oracle_lib):
    """Particle cell indices (truncation and round indexing) identical."""
    p, s, ref, nsteps, _ = load("heated16_2steps")
    o = run_oracle(oracle_lib, p, s, nsteps)
    part = o.get_particles(0)
    for q, L, N in (("x", p.Lx, p.Nx), ("y", p.Ly, p.Ny), ("z", p.Lz, p.Nz)):
        idx = 1.0 / (L / N)
        a, b = part[q] * idx, ref["part"][q] * idx
        assert np.array_equal(a.astype(np.int64), b.astype(np.int64))
        assert np.array_equal(np.round(a), np.round(b))


def test_shipped_differs_from_patched(oracle_lib):
    """The shipped loop (particle stage commented out) is not the two-way
    coupled solver: its result differs from the patched one."""
    p, s, ref, nsteps, _ = load("shipped24_1step")
    a = run_oracle(oracle_lib, p, s, 1, with_particles=False).get_field("RU")
    b = run_oracle(oracle_lib, p, s, 1, with_particles=True).get_field("RU")
    assert rel_err(a, b) > 1e-6


@pytest.mark.parametrize("seed,N,steps,heat", [(101, 16, 3, 0.5), (102, 12, 2, 0.0)])
def test_oracle_matches_fresh_reference_run(oracle_lib, seed, N, steps, heat):
    if not oracle_lib.have_reference():
        pytest.skip("reference sources not present on this machine")
    npart = 800
    p = P.physical(N, npart, nu=0.02, A=0.1, tau_p=0.1, mass_loading=0.4, heating_Q=heat,
                   iterations=4, epsilon=0.0)
    s = inputs.make_state(p, npart, seed=seed)
    p = p.replace(dt=inputs.cfl_dt(p, s.RU))
    ref = oracle_lib.run_reference(p, s, steps)
    o = run_oracle(oracle_lib, p, s, steps)
    compare(o, {"RU": ref["RU"], "RU_int": ref["RU_int"], "Rho": ref["Rho"], "P": ref["P"],
                "part": ref["part"]}, TOL)
    assert rel_err(o.get_field("C"), ref["C"]) <= TOL
    assert rel_err(o.get_field("Q"), ref["RHS_Part_Temp"]) <= 1e-11


@pytest.mark.parametrize("name", SCALAR_NAMES)
def test_oracle_passive_scalar_matches_golden(oracle_lib, name):
    """Passive scalar transport (grid.cpp:743-772) with each source type."""
    p, s, ref, nsteps, _ = load(name)
    o = run_oracle(oracle_lib, p, s, nsteps)
    compare(o, ref, TOL)
    assert rel_err(o.get_field("PASSIVE_SCALAR"), ref["PS"]) <= TOL
    assert rel_err(ref["PS"], s.PS) > 1e-3  # the scalar did move
