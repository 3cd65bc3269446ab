"""Parity of the GPU path (libtpm.so, called through the C ABI) with the
oracle and with the reference's own outputs.

Tolerances (FP64 path): <= 1e-12 relative per field after one RK4 step,
<= 1e-9 after ten; particle cell indices identical.  The relative error of a
field is max|a-b| / max|b|.  The heat exchange rate is a difference of nearly
equal temperatures, so it is held to 1e-11 relative (its absolute error is
at roundoff of the temperatures).
"""
import numpy as np
import pytest

from conftest import rel_err
from golden import NAMES, load
from tpm import inputs, params as P

pytestmark = pytest.mark.gpu

TOL1 = 1e-12
TOL10 = 1e-9


@pytest.fixture(scope="module")
def capi():
    from tpm import build, capi

    build.build()
    return capi


def gpu_run(capi, p, s, nsteps=0, substeps=None, tau=None):
    ctx = capi.Context(p, s.npart)
    ctx.set_option(capi.OPT_STORE_DIVERGENCE, 1)
    ctx.load(s)
    if tau is not None:
        ctx.set_tau(tau)
    ctx.initialize()
    if substeps is not None:
        for k in range(substeps):
            ctx.substep(k)
    else:
        ctx.run(nsteps)
    ctx.sync()
    return ctx


def oracle_run(oracle_lib, p, s, nsteps=0, substeps=None, tau=None):
    o = oracle_lib.Oracle(p, s.npart)
    o.load(s)
    if tau is not None:
        o.set_tau(tau)
    o.initialize()
    if substeps is not None:
        for k in range(substeps):
            o.substep(k)
    else:
        for _ in range(nsteps):
            o.step()
    return o


def make_case(N, npart, seed, heat=0.3, iterations=3, eps=0.0, mass_loading=0.5, **extra):
    p = P.physical(N, npart, nu=0.02, A=0.1, tau_p=0.1, mass_loading=mass_loading,
                   heating_Q=heat, iterations=iterations, epsilon=eps)
    s = inputs.make_state(p, npart, seed=seed)
    p = p.replace(dt=inputs.cfl_dt(p, s.RU), **extra)
    return p, s


FIELDS = [("RU", "RU"), ("RU_INT", "RU_INT"), ("RHO", "RHO"), ("P", "P"), ("C", "C")]


def assert_state_close(ctx, o, tol, check_rhs_t=True, check_q=True):
    """check_q / check_rhs_t: with heating off the particle heat exchange is
    (Tg - T_p) of two temperatures equal up to roundoff, so it is roundoff
    noise and has no meaningful relative error."""
    for g, r in FIELDS:
        a = ctx.download_field(g)
        assert np.all(np.isfinite(a)), g
        e = rel_err(a, o.get_field(r))
        assert e <= tol, (g, e)
    if check_q:
        e = rel_err(ctx.download_field("Q"), o.get_field("Q"))
        assert e <= 10 * tol, ("Q", e)
    a, b = ctx.download_particles("base"), o.get_particles(0)
    assert np.array_equal(a["flag"], b["flag"])
    for q in inputs.PQ:
        e = rel_err(a[q], b[q])
        assert e <= tol, (q, e)
    if check_rhs_t:
        e = rel_err(ctx.download_rhs_t(), o.get_rhs_t())
        assert e <= 10 * tol, ("RHS_T", e)
    sg, so = ctx.scalars(), o.scalars()
    assert abs(sg["P0"] - so["P0"]) <= tol * abs(so["P0"])
    assert sg["T_cur"] == so["T_cur"]


# ------------------------------------------------------------------ goldens
@pytest.mark.parametrize("name", [n for n in NAMES if not n.startswith("shipped")])
def test_gpu_matches_reference_golden(capi, name):
    p, s, ref, nsteps, _ = load(name)
    ctx = gpu_run(capi, p, s, nsteps)
    for g, r in (("RU", "RU"), ("RU_INT", "RU_int"), ("RHO", "Rho"), ("P", "P"), ("C", "C")):
        e = rel_err(ctx.download_field(g), ref[r])
        assert e <= TOL1, (g, e)
    assert rel_err(ctx.download_field("Q"), ref["Q"]) <= 10 * TOL1
    part = ctx.download_particles("base")
    assert np.array_equal(part["flag"], ref["part"]["flag"])
    for q in inputs.PQ:
        assert rel_err(part[q], ref["part"][q]) <= TOL1, q
    assert abs(ctx.scalars()["P0"] - ref["P0"]) <= 1e-13 * abs(ref["P0"])


# ------------------------------------------------------------- substep level
@pytest.mark.parametrize("N,npart,stages", [(16, 500, 1), (24, 700, 2), (16, 300, 4)])
def test_substeps_match_oracle(capi, oracle_lib, N, npart, stages):
    p, s = make_case(N, npart, seed=N + stages)
    ctx = gpu_run(capi, p, s, substeps=stages)
    o = oracle_run(oracle_lib, p, s, substeps=stages)
    for g in ("RU_INT", "RU_NP1", "RHO_INT", "RHO_NP1", "P", "FP", "C", "RHS_POIS",
              "DIVERGENCE"):
        e = rel_err(ctx.download_field(g), o.get_field(g))
        assert e <= TOL1, (g, e)
    for pset, oset in (("int", 1), ("np1", 3)):
        a, b = ctx.download_particles(pset), o.get_particles(oset)
        for q in inputs.PQ:
            assert rel_err(a[q], b[q]) <= TOL1, (pset, q)


def test_initialize_heat_coupling(capi, oracle_lib):
    p, s = make_case(16, 800, seed=5, heat=1.0)
    s.part["T"] = 1.0 + 0.1 * np.sin(np.arange(s.npart))  # particles off equilibrium
    ctx = gpu_run(capi, p, s, substeps=0)
    o = oracle_run(oracle_lib, p, s, substeps=0)
    assert rel_err(ctx.download_field("Q"), o.get_field("Q")) <= 1e-13
    assert rel_err(ctx.download_rhs_t(), o.get_rhs_t()) <= 1e-13


# ----------------------------------------------------------- step level
def test_one_and_ten_steps_box32(capi, oracle_lib):
    """The CPU-runnable workload shape (32^3, 10^4 particles, two-way)."""
    p = P.physical(32, 10_000, nu=0.02, A=0.1, tau_p=0.1, mass_loading=0.2, heating_Q=0.0)
    s = inputs.make_state(p, 10_000, seed=0)
    p = p.replace(dt=inputs.cfl_dt(p, s.RU))
    ctx = gpu_run(capi, p, s, 1)
    o = oracle_run(oracle_lib, p, s, 1)
    assert_state_close(ctx, o, TOL1, check_rhs_t=False, check_q=False)
    ctx.run(9)
    ctx.sync()
    for _ in range(9):
        o.step()
    assert_state_close(ctx, o, TOL10, check_rhs_t=False, check_q=False)
    # particle cell indices identical (truncation and round indexing)
    a, b = ctx.download_particles("base"), o.get_particles(0)
    for q, L, N in (("x", p.Lx, p.Nx), ("y", p.Ly, p.Ny), ("z", p.Lz, p.Nz)):
        idx = 1.0 / (L / N)
        assert np.array_equal((a[q] * idx).astype(np.int64), (b[q] * idx).astype(np.int64))
        assert np.array_equal(np.round(a[q] * idx), np.round(b[q] * idx))


def test_heated_tolerance_controlled_poisson(capi, oracle_lib):
    """Variable density (heating on) with the reference's own stopping rule."""
    p, s = make_case(24, 2000, seed=9, heat=2.0, iterations=20, eps=1e-13)
    ctx = gpu_run(capi, p, s, 2)
    o = oracle_run(oracle_lib, p, s, 2)
    assert_state_close(ctx, o, TOL1)
    assert ctx.scalars()["last_poisson_iterations"] >= 2


def test_anisotropic_box_and_options(capi, oracle_lib):
    """Nx != Ny != Nz, Lx != Ly != Lz, gravity, cooling and the threshold switch."""
    p, s = make_case(16, 600, seed=21, heat=0.5)
    p = p.replace(Nx=20, Ny=12, Nz=18, Lx=1.3 * p.Lx, Lz=0.8 * p.Lz)
    s = inputs.make_state(p, 600, seed=21)
    p = p.replace(dt=inputs.cfl_dt(p, s.RU), cooling=1, ParticleGravity=1, gx1=0.3, gz1=-0.4,
                  gx2=-0.2, gz2=-0.8, A2=0.3, I02=2 * p.I01, threshold=1.5 * p.dt, Iteration2=4)
    ctx = gpu_run(capi, p, s, 3)
    o = oracle_run(oracle_lib, p, s, 3)
    assert_state_close(ctx, o, TOL1)


def test_polydisperse_stokes_times(capi, oracle_lib):
    p, s = make_case(16, 1500, seed=31)
    tau = inputs.log_uniform_tau(s.npart, 0.05, 0.5, seed=31)
    ctx = gpu_run(capi, p, s, 2, tau=tau)
    o = oracle_run(oracle_lib, p, s, 2, tau=tau)
    assert_state_close(ctx, o, TOL1)


# ------------------------------------------------------------- edge cases
def test_no_particles(capi, oracle_lib):
    p, s = make_case(16, 10, seed=3)
    s.part = {k: v[:0] for k, v in s.part.items()}
    ctx = gpu_run(capi, p, s, 2)
    o = oracle_run(oracle_lib, p, s, 2)
    for g in ("RU", "RHO", "P"):
        assert rel_err(ctx.download_field(g), o.get_field(g)) <= TOL1
    assert np.abs(ctx.download_field("C")).max() == 0


def test_boundary_and_clustered_particles(capi, oracle_lib):
    """Particles on cell faces, at 0, next to L, and many in one cell.  (Mass
    loading small enough that 40 coincident particles do not make the coupled
    system blow up - with 0.5 it diverges in the oracle as well.)"""
    p, s = make_case(16, 64, seed=4, mass_loading=2e-3)
    L, dx = p.Lx, p.dx
    x = np.concatenate([np.zeros(8), np.full(8, np.nextafter(L, 0)), np.arange(8) * dx,
                        np.full(40, 3.3 * dx)])
    part = s.part
    for q, arr in (("x", x), ("y", np.roll(x, 5)), ("z", np.roll(x, 11))):
        part[q] = arr.copy()
    part["u"] = np.linspace(-1, 1, 64)  # some leave through either side
    part["v"] = -part["u"]
    ctx = gpu_run(capi, p, s, 2)
    o = oracle_run(oracle_lib, p, s, 2)
    assert_state_close(ctx, o, TOL1)
    a = ctx.download_particles("base")
    for q in ("x", "y", "z"):
        assert np.all(a[q] >= 0) and np.all(a[q] <= L)


def test_crowded_cell_matches_oracle(capi, oracle_lib):
    """200 coincident particles in one cell: the counting sort orders that
    cell's particles by a heap sort instead of the insertion sort of the usual
    few, and the deposits still sum in particle order like the oracle's."""
    p, s = make_case(16, 300, seed=6, mass_loading=1e-3)
    part = s.part
    for q, v in (("x", 5.4), ("y", 2.2), ("z", 9.7)):
        part[q][:200] = v * p.dx
    ctx = gpu_run(capi, p, s, 2)
    o = oracle_run(oracle_lib, p, s, 2)
    assert_state_close(ctx, o, TOL1)
    assert ctx.scalars()["num_timestep"] == 2  # no crowded-cell error below 65536


def test_single_particle(capi, oracle_lib):
    p, s = make_case(12, 1, seed=6, mass_loading=1e-4)
    ctx = gpu_run(capi, p, s, 3)
    o = oracle_run(oracle_lib, p, s, 3)
    assert_state_close(ctx, o, TOL1)


# ------------------------------------------------------------- operators
@pytest.mark.parametrize("N", [16, 24, 30])
def test_poisson_operator_matches_oracle(capi, oracle_lib, N):
    p = P.physical(N, 1, nu=0.02, A=0.0, tau_p=0.1, mass_loading=0.1)
    rng = np.random.default_rng(N)
    C3 = 1.0 / (1.0 + 0.2 * rng.random((3, N, N, N)))
    RHS = rng.standard_normal((N, N, N))
    RHS -= RHS.mean()
    P0 = rng.standard_normal((N, N, N))
    ctx = capi.Context(p, 1)
    Pg, itg, errg = ctx.poisson_solve(C3, P0, RHS, 6, 0.0)
    o = oracle_lib.Oracle(p, 1)
    Po, ito, erro = o.poisson_solve(C3, P0, RHS, 6, 0.0)
    assert itg == ito == 6
    assert rel_err(Pg, Po) <= 1e-12
    assert abs(errg - erro) <= 1e-12 * max(abs(erro), 1e-300) + 1e-15


def test_deterministic_rerun(capi):
    p, s = make_case(24, 3000, seed=8)
    a = gpu_run(capi, p, s, 2)
    b = gpu_run(capi, p, s, 2)
    for g in ("RU", "RHO", "P", "C", "Q", "FP"):
        assert np.array_equal(a.download_field(g), b.download_field(g)), g


# ---------------------------------------------- size-independent properties
def test_large_box_properties(capi):
    """128^3 with 2e5 particles: after a step the projected velocity satisfies
    the discrete divergence constraint, density mass is conserved, the mean
    momentum equals the prescribed value, and particles stay in the box."""
    N, npart = 128, 200_000
    p = P.physical(N, npart, nu=0.005, A=0.1, tau_p=0.1, mass_loading=0.5, heating_Q=0.1,
                   iterations=20, epsilon=1e-13)
    s = inputs.make_state(p, npart, seed=1)
    p = p.replace(dt=inputs.cfl_dt(p, s.RU))
    ctx = gpu_run(capi, p, s, substeps=1)
    # after stage 0: div(RU_new/Rho_face) equals the divergence constraint up
    # to a constant (the discrete divergence has zero mean; the constraint's
    # mean is carried by dP0/dt, grid.cpp:822,848)
    RUn = ctx.download_field("RU_INT")
    Rn = ctx.download_field("RHO_INT")
    div_target = ctx.download_field("DIVERGENCE")
    Rf = [(Rn + np.roll(Rn, 1, axis=2 - d)) * 0.5 for d in range(3)]
    U = np.stack([RUn[d] / Rf[d] for d in range(3)])
    r = inputs.div_f2c(p, U) - div_target
    r -= r.mean()
    assert np.abs(r).max() <= 1e-9 * np.abs(div_target).max() + 1e-9
    m0 = s.Rho.sum()
    ctx.substep(1)
    ctx.substep(2)
    ctx.substep(3)
    ctx.end_step()
    assert abs(ctx.download_field("RHO").sum() - m0) <= 1e-12 * m0
    RU = ctx.download_field("RU")
    assert np.abs(RU.reshape(3, -1).mean(axis=1)).max() <= 1e-13
    part = ctx.download_particles("base")
    for q, L in (("x", p.Lx), ("y", p.Ly), ("z", p.Lz)):
        assert part[q].min() >= 0 and part[q].max() <= L
    assert np.all(np.isfinite(RU))


def test_host_round_trip_resume_is_exact(capi):
    """Downloading the step-boundary state and resuming from it in a fresh
    context continues the run bit for bit (the e2e bench relies on this)."""
    p, s = make_case(24, 2000, seed=12, heat=0.5)
    a = gpu_run(capi, p, s, 2)
    st = a.download_state()
    a.run(2)
    a.sync()
    b = capi.Context(p, s.npart)
    b.upload_state(st)
    b.run(2)
    b.sync()
    for g in ("RU", "RU_INT", "RHO", "P", "Q", "C"):
        assert np.array_equal(a.download_field(g), b.download_field(g)), g
    pa, pb = a.download_particles("base"), b.download_particles("base")
    for q in inputs.PQ:
        assert np.array_equal(pa[q], pb[q]), q
    assert a.scalars()["P0"] == b.scalars()["P0"]
