"""The mixed-precision path (TPM_PREC_MIXED): FP32 right-hand-side stencil and
FP32 FFT correction solves on an FP64 state with FP64 residuals.

Bars: <= 1e-5 relative per field against the FP64 oracle (and the FP64 GPU
path) after 1 and 10 RK4 steps, and a post-projection FP64 divergence
residual max|div u - divergence| <= 1e-10.
"""
import numpy as np
import pytest

from conftest import rel_err
from tpm import inputs, params as P

pytestmark = pytest.mark.gpu

TOL_MIXED = 1e-5
TOL_DIV = 1e-10


@pytest.fixture(scope="module")
def capi():
    from tpm import build, capi

    build.build()
    return capi


def setup(N, npart, seed, heat, precision, **kw):
    p = P.physical(N, npart, nu=kw.get("nu", 0.02), A=0.1, tau_p=0.1,
                   mass_loading=kw.get("phi", 0.5), heating_Q=heat, iterations=20,
                   epsilon=1e-13, precision=precision)
    s = inputs.make_state(p, npart, seed=seed)
    p = p.replace(dt=inputs.cfl_dt(p, s.RU))
    return p, s


def run(capi, p, s, nsteps):
    ctx = capi.Context(p, s.npart)
    ctx.load(s)
    ctx.initialize()
    ctx.run(nsteps)
    ctx.sync()
    return ctx


@pytest.mark.parametrize("heat", [0.0, 0.5])
def test_mixed_matches_fp64_oracle(capi, oracle_lib, heat):
    p, s = setup(32, 10_000, seed=5, heat=heat, precision=P.PREC_MIXED)
    ctx = run(capi, p, s, 1)
    o = oracle_lib.Oracle(p, s.npart)
    o.load(s)
    o.initialize()
    o.step()

    def check():
        for g in ("RU", "RU_INT", "RHO", "P"):
            e = rel_err(ctx.download_field(g), o.get_field(g))
            assert e <= TOL_MIXED, (g, e)
        a, b = ctx.download_particles("base"), o.get_particles(0)
        for q in inputs.PQ:
            assert rel_err(a[q], b[q]) <= TOL_MIXED, q
        sc = ctx.scalars()
        assert sc["max_abs_div"] >= 0 and sc["max_abs_div"] <= TOL_DIV, sc["max_abs_div"]
        assert abs(sc["P0"] - o.scalars()["P0"]) <= TOL_MIXED

    check()
    ctx.run(9)
    ctx.sync()
    for _ in range(9):
        o.step()
    check()


def test_mixed_matches_fp64_gpu_128(capi):
    """Heated 128^3 box with 10^6 particles: mixed vs FP64 GPU after 1 and 10
    steps, per field and per particle quantity, and no particle in another
    gas-velocity cell (truncated index) than on the FP64 path."""
    p, s = setup(128, 1_000_000, seed=1, heat=0.1, precision=P.PREC_MIXED, nu=0.005)
    ctxs = []
    for prec in (P.PREC_MIXED, P.PREC_FP64):
        c = capi.Context(p.replace(precision=prec), s.npart)
        c.load(s)
        c.initialize()
        ctxs.append(c)
    m, f = ctxs
    for more in (1, 9):
        for c in ctxs:
            c.run(more)
            c.sync()
        for g in ("RU", "RHO", "P", "C", "Q"):
            e = rel_err(m.download_field(g), f.download_field(g))
            assert e <= TOL_MIXED, (g, e)
        assert m.scalars()["max_abs_div"] <= TOL_DIV
        pm, pf = m.download_particles("base"), f.download_particles("base")
        for q in inputs.PQ:
            assert rel_err(pm[q], pf[q]) <= TOL_MIXED, q
        for q, L, n in (("x", p.Lx, p.Nx), ("y", p.Ly, p.Ny), ("z", p.Lz, p.Nz)):
            idx = n / L
            assert np.array_equal(np.trunc(pm[q] * idx), np.trunc(pf[q] * idx)), q


def test_mixed_matches_fp64_on_ragged_tiles(capi):
    """A box whose sides are not multiples of the z-marching kernels' 32 x 8
    column tiles and whose Nz is not a multiple of their z chunk: mixed vs
    FP64 GPU after 3 heated steps."""
    p, s = setup(24, 6000, seed=9, heat=0.5, precision=P.PREC_MIXED)
    p = p.replace(Ny=20, Nz=18, Ly=p.Lx * 20 / 24, Lz=p.Lx * 18 / 24)
    s = inputs.make_state(p, s.npart, seed=9)
    p = p.replace(dt=inputs.cfl_dt(p, s.RU))
    m = run(capi, p, s, 3)
    f = run(capi, p.replace(precision=P.PREC_FP64), s, 3)
    for g in ("RU", "RHO", "P", "C", "Q"):
        e = rel_err(m.download_field(g), f.download_field(g))
        assert e <= TOL_MIXED, (g, e)
    assert m.scalars()["max_abs_div"] <= TOL_DIV
    pm, pf = m.download_particles("base"), f.download_particles("base")
    for q in inputs.PQ:
        assert rel_err(pm[q], pf[q]) <= TOL_MIXED, q


@pytest.mark.parametrize("shape", [(32, 32, 256), (32, 256, 32)])
def test_mixed_matches_fp64_with_256_point_pencils(capi, shape):
    """Boxes with 256-point z (or y) pencils, the size whose z pass runs its
    second forward stage, the divide and the first inverse stage in registers:
    mixed vs FP64 GPU after 1 and 3 heated steps."""
    nx, ny, nz = shape
    p, s = setup(nx, 20_000, seed=13, heat=0.5, precision=P.PREC_MIXED)
    p = p.replace(Ny=ny, Nz=nz, Ly=p.Lx * ny / nx, Lz=p.Lx * nz / nx)
    s = inputs.make_state(p, s.npart, seed=13)
    p = p.replace(dt=inputs.cfl_dt(p, s.RU))
    ctxs = []
    for prec in (P.PREC_MIXED, P.PREC_FP64):
        c = capi.Context(p.replace(precision=prec), s.npart)
        c.load(s)
        c.initialize()
        ctxs.append(c)
    m, f = ctxs
    for more in (1, 2):
        for c in ctxs:
            c.run(more)
            c.sync()
        for g in ("RU", "RHO", "P", "C", "Q"):
            e = rel_err(m.download_field(g), f.download_field(g))
            assert e <= TOL_MIXED, (g, e)
        assert m.scalars()["max_abs_div"] <= TOL_DIV
        pm, pf = m.download_particles("base"), f.download_particles("base")
        for q in inputs.PQ:
            assert rel_err(pm[q], pf[q]) <= TOL_MIXED, q


def test_mixed_keeps_the_callers_particle_order(capi):
    """The mixed path keeps its particles in cell order in memory (a
    permutation at every step boundary); every transfer is in the caller's
    order: flags come back unchanged, per-particle Stokes times stay with
    their particles, and each particle matches the FP64 path's."""
    p, s = setup(32, 5000, seed=11, heat=0.5, precision=P.PREC_MIXED)
    rng = np.random.default_rng(5)
    s.part["flag"] = rng.permutation(s.npart).astype(np.int32)
    tau = rng.uniform(0.05, 0.2, s.npart)
    out = []
    for prec in (P.PREC_MIXED, P.PREC_FP64):
        ctx = capi.Context(p.replace(precision=prec), s.npart)
        ctx.load(s)
        ctx.set_tau(tau)
        ctx.initialize()
        ctx.run(4)
        ctx.sync()
        out.append((ctx.download_particles("base"), ctx.download_rhs_t()))
    (pm, rm), (pf, rf) = out
    assert np.array_equal(pm["flag"], s.part["flag"])
    for q in inputs.PQ:
        assert rel_err(pm[q], pf[q]) <= TOL_MIXED, q
        assert np.abs(pm[q] - pf[q]).max() <= 1e-4 * np.abs(pf[q]).max(), q
    assert rel_err(rm, rf) <= TOL_MIXED


def test_mixed_restart_and_state_transfer_in_callers_order(capi, tmp_path):
    """Restart files and the step-boundary state carry the caller's particle
    order on the mixed path, whose particles sit in cell order in memory:
    after 3 steps both hold exactly what download_particles returns; a fresh
    context reading the files gives them back unchanged and steps on like a
    context loaded from the same arrays; and a context loaded with
    tpm_load_state continues like the first run.  Mixed runs whose inputs
    differ in rounding (here the in-cell order of the deposit sums, since a
    fresh context's particles start in the caller's order) part at the level
    of their FP32 increments, 1e-8 to 1e-7 after two steps (held to 1e-6); a
    wrong particle order would show as an O(1) difference."""
    p, s = setup(32, 6000, seed=13, heat=0.5, precision=P.PREC_MIXED)
    a = run(capi, p, s, 3)
    d = str(tmp_path)
    a.write_restart(d)
    r = inputs.read_restart(d, p)
    st = a.download_state()
    base = a.download_particles("base")
    for q in inputs.PQ + ("flag",):
        assert np.array_equal(r.part[q], base[q]), q
    for q in inputs.PQ:
        assert np.array_equal(st["part"][q], base[q]), q
    b = capi.Context(p, s.npart)
    b.read_restart(d)
    back = b.download_particles("base")
    for q in inputs.PQ:
        assert np.array_equal(back[q], base[q]), q
    b.initialize()
    b2 = capi.Context(p, s.npart)
    b2.load(r)
    b2.initialize()
    c = capi.Context(p, s.npart)
    c.upload_state(st)
    for ctx in (a, b, b2, c):
        ctx.run(2)
        ctx.sync()
    for x, y in ((b, b2), (c, a)):
        for g in ("RU", "RHO", "P", "C", "Q"):
            assert rel_err(x.download_field(g), y.download_field(g)) <= 1e-6, g
        px, py = x.download_particles("base"), y.download_particles("base")
        for q in inputs.PQ:
            assert rel_err(px[q], py[q]) <= 1e-6, q


@pytest.mark.parametrize("graph", [False, True])
def test_divergence_residual_on_read_equals_in_step(capi, graph):
    """The last stage's post-projection residual, evaluated when the scalars
    are first read after a step, equals the one the every-stage option
    evaluates inside the step (same kernel, same inputs), the fields stay
    bit-identical, and a read after a field upload keeps the last value."""
    p, s = setup(24, 4000, seed=17, heat=0.5, precision=P.PREC_MIXED)
    ctxs = []
    for every in (False, True):
        c = capi.Context(p, s.npart)
        c.set_graph(graph)
        if every:
            c.set_option(capi.OPT_DIV_RESIDUAL_EVERY_STAGE, 1)
        c.load(s)
        c.initialize()
        ctxs.append(c)
    lazy, eager = ctxs
    for more in (1, 2):
        for c in ctxs:
            c.run(more)
            c.sync()
        a, b = lazy.scalars()["max_abs_div"], eager.scalars()["max_abs_div"]
        assert 0 < a <= TOL_DIV and a == b, (a, b)
        for g in ("RU", "RU_INT", "RHO", "P", "C", "Q"):
            assert np.array_equal(lazy.download_field(g), eager.download_field(g)), g
    kept = lazy.scalars()["max_abs_div"]
    lazy.upload_field("RU_INT", lazy.download_field("RU_INT") * 1.01)
    assert lazy.scalars()["max_abs_div"] == kept


@pytest.mark.parametrize("graph", [False, True])
def test_fused_deposits_match_two_pass(capi, graph):
    """The heat/concentration and the momentum deposits in one z-marching pass
    each (grids of whole 32 x 8 tiles) give the bits of the two-pass deposits:
    Q of the initial deposit, and the concentration and the momentum source of
    the first stage.  Later the runs part only by the rounding of the heat
    total's per-block sums (which feed the P0 update), held to 1e-12."""
    p, s = setup(32, 20_000, seed=19, heat=0.5, precision=P.PREC_MIXED)
    ctxs = []
    for fused in (1, 0):
        c = capi.Context(p, s.npart)
        c.set_graph(graph)
        c.set_option(capi.OPT_FUSED_DEPOSITS, fused)
        c.load(s)
        c.initialize()
        ctxs.append(c)
    a, b = ctxs
    assert np.array_equal(a.download_field("Q"), b.download_field("Q"))
    for c in ctxs:
        c.substep(0)
        c.sync()
    for g in ("FP", "C"):
        assert np.array_equal(a.download_field(g), b.download_field(g)), g
    for c in ctxs:
        for st in (1, 2, 3):
            c.substep(st)
        c.end_step()
        c.run(2)
        c.sync()
    for g in ("RU", "RHO", "P", "C", "Q"):
        assert rel_err(a.download_field(g), b.download_field(g)) <= 1e-12, g
    pa, pb = a.download_particles("base"), b.download_particles("base")
    for q in inputs.PQ:
        assert rel_err(pa[q], pb[q]) <= 1e-12, q
