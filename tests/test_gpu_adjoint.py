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


# ------------------------------------------- the 64^3 workload of the adjoint
def case64(iterations=4):
    """64^3 cells and 2e5 two-way-coupled particles (nu = 0.01, A = 0.1,
    Stokes time 0.1, mass loading 0.3, seed 3).  The finite-difference checks
    run a fixed number of Richardson iterations per solve (epsilon = 0): a
    tolerance-controlled loop makes J piecewise in its inputs (the stopping
    iteration can change with the perturbation), which the adjoint, like any
    derivative, does not see."""
    p = P.physical(64, 200_000, nu=0.01, A=0.1, tau_p=0.1, mass_loading=0.3, heating_Q=0.0,
                   iterations=iterations, epsilon=0.0)
    s = inputs.make_state(p, 200_000, seed=3)
    s.tau = np.full(s.npart, 0.1)
    return p.replace(dt=inputs.cfl_dt(p, s.RU)), s


def test_adjoint_64_matches_the_reference_gradient(capi, oracle_lib):
    """64^3 cells, 2e5 particles, a 10-step horizon, checkpoints every 4 steps:
    J and the gradients of J = TKE + var(C) with respect to the initial
    momentum, A and tau_p against the FP64 reference gradient of the CPU
    restatement (oracle/adjoint_ref.py), which follows the same trajectory."""
    import adjoint_ref as ar

    p, s = case64()
    ctx, J, g, gA, gt = gpu_grad(capi, p, s, 10, 1.0, 1.0, K=4)
    s_ref = inputs.State(RU=s.RU, Rho=s.Rho, P=s.P, part=s.part, P0=s.P0)
    Jr, gr, gAr, gtr = ar.gradient(p, s_ref, 10, 1.0, 1.0, oracle_lib, tau=0.1)
    assert abs(J - Jr) <= 1e-12 * abs(Jr)
    assert rel_err(g, gr) <= 1e-9
    assert abs(gA - gAr) <= 1e-9 * abs(gAr)
    assert abs(gt - gtr) <= 1e-9 * abs(gtr)


def test_adjoint_64_matches_finite_differences_in_16_directions(capi):
    """J = TKE + var(C) at 64^3 + 2e5 particles over a 3-step horizon: the
    gradient with respect to the initial momentum against central differences
    (h = 1e-6) along 16 random discretely divergence-free directions, and
    dJ/dA and dJ/dtau_p against theirs, within 1e-6 of the largest directional
    derivative.

    The discrete J is only piecewise smooth: the reference's gas velocity at a
    particle is nearest-cell across the faces transverse to each component
    (particle.cpp:340-360), so a perturbation that moves one particle across
    such a face at a stage evaluation makes J jump (by ~5e-8 here, i.e. ~2e-2
    in a difference quotient with h = 1e-6).  Over 10 steps the +-h runs of a
    direction straddle several such jumps; over 3 steps few do.  A pair whose
    final particle positions differ by more than 1e-7 somewhere (a smooth
    response moves them by ~1e-9) straddled a jump and is retried with
    h = 1e-8; at most 2 of the 16 directions may straddle one at both h.
    The derivative the adjoint gives is the one of the smooth branch, which
    the 10-step comparison with the reference gradient checks everywhere."""
    import adjoint_ref as ar

    p, s = case64()
    nsteps, w_tke, w_cvar = 3, 1.0, 1.0
    ctx, J, g, gA, gt = gpu_grad(capi, p, s, nsteps, w_tke, w_cvar, K=2)

    def run(RU=s.RU, A=p.A1, tau=0.1):
        c = capi.Context(p.replace(A1=A, A2=A), s.npart)
        st = inputs.State(RU=RU, Rho=s.Rho, P=s.P, part=s.part, P0=s.P0,
                          tau=np.full(s.npart, tau))
        c.load(st)
        c.initialize()
        c.run(nsteps)
        part = c.download_particles()
        X = np.stack([part[q] for q in ("x", "y", "z")])
        out = ar.objective(p, c.download_field("RU"), c.download_field("RHO"), X, w_tke, w_cvar)
        c.close()
        return out, X

    def central(perturbed):
        for h in (1e-6, 1e-8):
            (jp, xp), (jm, xm) = perturbed(h), perturbed(-h)
            if np.abs(xp - xm).max() <= 1e-7:  # no jump between the two runs
                return (jp - jm) / (2 * h)
        return None

    assert abs(run()[0] - J) <= 1e-12 * abs(J)
    fd, ad = [], []
    for seed in range(100, 116):
        v = inputs.solenoidal_velocity(p, seed)
        fd.append(central(lambda h: run(RU=s.RU + h * v)))
        ad.append(float(np.sum(g * v)))
    ok = [i for i, f in enumerate(fd) if f is not None]
    assert len(ok) >= 14, f"{16 - len(ok)} directions straddle a jump of J"
    scale = max(abs(a) for a in ad)
    for i in ok:
        assert abs(fd[i] - ad[i]) <= 1e-6 * scale, (i, fd[i], ad[i])
    fdA = central(lambda h: run(A=p.A1 + h))
    fdt = central(lambda h: run(tau=0.1 + h))
    assert fdA is not None and fdt is not None
    assert abs(fdA - gA) <= 1e-6 * abs(fdA), (fdA, gA)
    assert abs(fdt - gt) <= 1e-6 * abs(fdt), (fdt, gt)


def test_adjoint_64_ten_steps_against_small_step_differences(capi):
    """The 10-step horizon at 64^3 + 2e5 particles: with h = 1e-6 the +-h runs
    of every direction straddle jumps of J (about 1000-2000 particles end
    1e-5-1e-4 apart instead of ~1e-8, and the difference quotients are off by
    up to 80 %); with h = 1e-8 no particle jumps and the central differences
    along 16 divergence-free directions match the adjoint within 1e-6 of the
    largest directional derivative (their own rounding is ~1e-7)."""
    import adjoint_ref as ar

    p, s = case64()
    nsteps, h = 10, 1e-8
    ctx, J, g, gA, gt = gpu_grad(capi, p, s, nsteps, 1.0, 1.0, K=4)

    def run(RU):
        c = capi.Context(p, s.npart)
        st = inputs.State(RU=RU, Rho=s.Rho, P=s.P, part=s.part, P0=s.P0, tau=s.tau)
        c.load(st)
        c.initialize()
        c.run(nsteps)
        part = c.download_particles()
        X = np.stack([part[q] for q in ("x", "y", "z")])
        out = ar.objective(p, c.download_field("RU"), c.download_field("RHO"), X, 1.0, 1.0)
        c.close()
        return out, X

    fd, ad = [], []
    for seed in range(100, 116):
        v = inputs.solenoidal_velocity(p, seed)
        (jp, xp), (jm, xm) = run(s.RU + h * v), run(s.RU - h * v)
        assert np.abs(xp - xm).max() <= 1e-7, seed  # no jump between the two runs
        fd.append((jp - jm) / (2 * h))
        ad.append(float(np.sum(g * v)))
    fd, ad = np.array(fd), np.array(ad)
    assert np.abs(fd - ad).max() <= 1e-6 * np.abs(ad).max(), (fd, ad)


def test_adjoint_64_over_the_200_step_horizon(capi):
    """The 200-step horizon of the adjoint workload (64^3 + 2e5 particles,
    Poisson loop as in the forward workload, checkpoints every 20 steps): J
    equals the plain forward run's, the gradients do not depend on the
    checkpoint interval (20 or 50 steps: recomputation is exact), and they are
    finite."""
    p, s = case64()
    p = p.replace(Iteration1=20, Iteration2=20, epsilon=1e-13)
    out = [gpu_grad(capi, p, s, 200, 1.0, 1.0, K=K)[1:] for K in (20, 50)]
    c = capi.Context(p, s.npart)
    c.load(s)
    c.initialize()
    c.run(200)
    import adjoint_ref as ar

    part = c.download_particles()
    X = np.stack([part[q] for q in ("x", "y", "z")])
    J_plain = ar.objective(p, c.download_field("RU"), c.download_field("RHO"), X, 1.0, 1.0)
    (J1, g1, gA1, gt1), (J2, g2, gA2, gt2) = out
    assert J1 == J2
    assert abs(J1 - J_plain) <= 1e-12 * abs(J_plain)
    assert np.all(np.isfinite(g1)) and np.isfinite(gA1) and np.isfinite(gt1)
    assert rel_err(g2, g1) <= 1e-13
    assert abs(gA2 - gA1) <= 1e-13 * abs(gA1) and abs(gt2 - gt1) <= 1e-13 * abs(gt1)
