"""The CPU reference gradient (oracle/adjoint_ref.py) against central finite
differences of the oracle: the discrete adjoint of the RK4 step in the
uniform-density two-way-coupled regime of the adjoint workload.

Directions: a random discretely divergence-free initial momentum
perturbation, the forcing coefficient A, and a uniform Stokes time.  Bar:
1e-6 relative (the finite differences themselves are good to ~1e-8 here).
"""
import numpy as np
import pytest

from tpm import inputs, params as P

TOL = 1e-6


@pytest.mark.parametrize("w_tke,w_cvar", [(1.0, 0.0), (0.0, 1.0), (1.0, 50.0)])
def test_reference_gradient_matches_finite_differences(oracle_lib, w_tke, w_cvar):
    import adjoint_ref as ar

    N, npart, nsteps, tau = 12, 60, 2, 0.1
    p = P.physical(N, npart, nu=0.05, A=0.1, tau_p=tau, mass_loading=0.3, iterations=3,
                   epsilon=0.0)
    s = inputs.make_state(p, npart, seed=3)
    p = p.replace(dt=inputs.cfl_dt(p, s.RU))
    J, gRU, gA, gtau = ar.gradient(p, s, nsteps, w_tke, w_cvar, oracle_lib, tau=tau)

    def J_of(RU=s.RU, A=p.A1, t=tau):
        st = inputs.State(RU=RU, Rho=s.Rho, P=s.P, part=s.part, P0=s.P0)
        return ar.forward_J(p.replace(A1=A, A2=A), st, nsteps, w_tke, w_cvar, oracle_lib, tau=t)

    assert abs(J_of() - J) <= 1e-14 * abs(J)
    h = 1e-6
    v = inputs.solenoidal_velocity(p, 99)
    checks = [
        ((J_of(RU=s.RU + h * v) - J_of(RU=s.RU - h * v)) / (2 * h), float(np.sum(gRU * v))),
        ((J_of(A=p.A1 + h) - J_of(A=p.A1 - h)) / (2 * h), gA),
        ((J_of(t=tau + h) - J_of(t=tau - h)) / (2 * h), gtau),
    ]
    for fd, ad in checks:
        assert abs(fd - ad) <= TOL * abs(fd), (fd, ad)
