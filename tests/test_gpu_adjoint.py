"""The discrete adjoint on the GPU (tpm_adjoint_run) against the CPU reference
gradient (oracle/adjoint_ref.py, itself checked against finite differences of
the oracle) and against central finite differences of the GPU forward run,
with checkpointed recomputation, and through a torch.autograd.Function.

Bars: J within 1e-12 of the reference; gradients within 1e-9 (relative to
their largest entry) of the reference; 1e-6 against finite differences.
"""
import numpy as np
import pytest

from conftest import rel_err
from tpm import inputs, params as P

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def capi():
    from tpm import build, capi

    build.build()
    return capi


def case(N=16, npart=300, nsteps=3, seed=3, tau=0.1):
    p = P.physical(N, npart, nu=0.03, A=0.1, tau_p=tau, mass_loading=0.3, iterations=3,
                   epsilon=0.0)
    s = inputs.make_state(p, npart, seed=seed)
    s.tau = np.full(npart, tau)
    return p.replace(dt=inputs.cfl_dt(p, s.RU)), s


def gpu_grad(capi, p, s, nsteps, w_tke, w_cvar, K=2):
    ctx = capi.Context(p, s.npart)
    ctx.load(s)
    ctx.initialize()
    J, g, gA, gt = ctx.adjoint(nsteps, checkpoint_every=K, w_tke=w_tke, w_cvar=w_cvar)
    return ctx, J, g, gA, gt


@pytest.mark.parametrize("w_tke,w_cvar", [(1.0, 0.0), (0.0, 1.0), (1.0, 30.0)])
def test_gpu_adjoint_matches_reference_gradient(capi, oracle_lib, w_tke, w_cvar):
    import adjoint_ref as ar

    p, s = case()
    nsteps = 3
    ctx, J, g, gA, gt = gpu_grad(capi, p, s, nsteps, w_tke, w_cvar)
    s_ref = inputs.State(RU=s.RU, Rho=s.Rho, P=s.P, part=s.part, P0=s.P0)
    Jr, gr, gAr, gtr = ar.gradient(p, s_ref, nsteps, w_tke, w_cvar, oracle_lib, tau=0.1)
    assert abs(J - Jr) <= 1e-12 * abs(Jr)
    assert rel_err(g, gr) <= 1e-9
    assert abs(gA - gAr) <= 1e-9 * abs(gAr)
    assert abs(gt - gtr) <= 1e-9 * abs(gtr)


def test_gpu_adjoint_matches_finite_differences_with_checkpoints(capi, oracle_lib):
    import adjoint_ref as ar

    p, s = case(N=24, npart=1500, nsteps=5, seed=4)
    nsteps, w_tke, w_cvar = 5, 1.0, 20.0
    ctx, J, g, gA, gt = gpu_grad(capi, p, s, nsteps, w_tke, w_cvar, K=2)

    def J_of(RU=s.RU, A=p.A1, tau=0.1):
        c = capi.Context(p.replace(A1=A, A2=A), s.npart)
        st = inputs.State(RU=RU, Rho=s.Rho, P=s.P, part=s.part, P0=s.P0,
                          tau=np.full(s.npart, tau))
        c.load(st)
        c.initialize()
        c.run(nsteps)
        part = c.download_particles()
        X = np.stack([part[q] for q in ("x", "y", "z")])
        return ar.objective(p, c.download_field("RU"), c.download_field("RHO"), X, w_tke, w_cvar)

    assert abs(J_of() - J) <= 1e-12 * abs(J)
    h = 1e-6
    v = inputs.solenoidal_velocity(p, 77)
    for fd, ad in (((J_of(RU=s.RU + h * v) - J_of(RU=s.RU - h * v)) / (2 * h), float(np.sum(g * v))),
                   ((J_of(A=p.A1 + h) - J_of(A=p.A1 - h)) / (2 * h), gA),
                   ((J_of(tau=0.1 + h) - J_of(tau=0.1 - h)) / (2 * h), gt)):
        assert abs(fd - ad) <= 1e-6 * abs(fd), (fd, ad)
    # the context is left at the final state of an ordinary run
    c = capi.Context(p, s.npart)
    c.load(s)
    c.initialize()
    c.run(nsteps)
    assert np.array_equal(ctx.download_field("RU"), c.download_field("RU"))
    assert np.array_equal(ctx.download_particles()["x"], c.download_particles()["x"])


def test_checkpoint_interval_does_not_change_the_gradient(capi):
    p, s = case(N=16, npart=400, nsteps=6, seed=5)
    out = [gpu_grad(capi, p, s, 6, 1.0, 10.0, K=K)[1:] for K in (1, 4, 6)]
    for J, g, gA, gt in out[1:]:
        assert J == out[0][0]
        assert rel_err(g, out[0][1]) <= 1e-13
        assert abs(gA - out[0][2]) <= 1e-13 * abs(out[0][2])
        assert abs(gt - out[0][3]) <= 1e-13 * abs(out[0][3])


def test_adjoint_refuses_heated_flow(capi):
    p, s = case()
    ctx = capi.Context(p.replace(I01=1.0, I02=1.0), s.npart)
    ctx.load(s)
    ctx.initialize()
    with pytest.raises(capi.TpmError):
        ctx.adjoint(1)


def test_torch_autograd_function(capi):
    torch = pytest.importorskip("torch")
    from torch_adjoint import TpmObjective

    p, s = case(N=16, npart=300, seed=6)
    RU0 = torch.tensor(s.RU, dtype=torch.float64, requires_grad=True)
    A = torch.tensor(p.A1, dtype=torch.float64, requires_grad=True)
    tau = torch.tensor(0.1, dtype=torch.float64, requires_grad=True)
    J = TpmObjective.apply(RU0, A, tau, capi, p, s, 3, 1.0, 10.0)
    (2.0 * J).backward()
    ctx, Jc, g, gA, gt = gpu_grad(capi, p, s, 3, 1.0, 10.0)
    assert abs(J.item() - Jc) <= 1e-12 * abs(Jc)
    assert rel_err(RU0.grad.numpy(), 2.0 * g) <= 1e-12
    assert abs(A.grad.item() - 2.0 * gA) <= 1e-12 * abs(gA)
    assert abs(tau.grad.item() - 2.0 * gt) <= 1e-12 * abs(gt)
