"""The 128^3 GPU-versus-CPU workload as specified: 128^3 cells, 10^6
two-way-coupled particles with Stokes times drawn log-uniform in [0.05, 0.5],
nu = 0.005, forcing A = 0.1, particle heating Q = 0.1 with two-way energy
coupling, Poisson stopping tolerance 1e-13 (Solver 0, up to 20 iterations).

One CPU oracle run (the C restatement of the reference's step,
grid.cpp:608-900 and particle.cpp:314-654, with the per-particle Stokes time
in update_velocity, particle.cpp:362-399) of 20 steps is shared by the tests
of this module; 20 steps are what the oracle runs in about two minutes on one
host core.  Bars:
  * FP64 path: <= 1e-12 relative per field after 1 step, <= 1e-9 after 10,
    particle cell indices identical (truncated and rounded);
  * statistics every 10 steps (TKE, dissipation, energy spectrum shells,
    cumulative RDF pair counts, concentration variance) within 2 % of the
    oracle's, for the FP64 and the mixed path;
  * mixed path: <= 1e-5 relative per field after 1 and 10 steps.
"""
import numpy as np
import pytest

from conftest import rel_err
from tpm import inputs, params as P

pytestmark = pytest.mark.gpu

N, NPART, SEED = 128, 1_000_000, 1
NSTEPS = 20        # oracle steps (statistics after 10 and 20)
TOL1, TOL10 = 1e-12, 1e-9
TOL_MIXED = 1e-5
TOL_STATS = 0.02
RDF_RMAX, RDF_BINS = 0.15, 15
FIELDS = ("RU", "RU_INT", "RHO", "P", "C")


def case(precision=P.PREC_FP64):
    p = P.physical(N, NPART, nu=0.005, A=0.1, tau_p=0.1, mass_loading=0.5, heating_Q=0.1,
                   iterations=20, epsilon=1e-13, precision=precision)
    s = inputs.make_state(p, NPART, seed=SEED)
    p = p.replace(dt=inputs.cfl_dt(p, s.RU))
    tau = inputs.log_uniform_tau(NPART, 0.05, 0.5, seed=SEED)
    return p, s, tau


def rdf_cumulative(p, part):
    """Cumulative pair counts of minimum-image distances below (b + 1) dr for
    the RDF bins, by a periodic k-d tree (the all-pairs count is O(Np^2))."""
    spatial = pytest.importorskip("scipy.spatial")
    L = np.array([p.Lx, p.Ly, p.Lz])
    pts = np.stack([part["x"], part["y"], part["z"]], axis=1) % L
    tree = spatial.cKDTree(pts, boxsize=L)
    r = RDF_RMAX / RDF_BINS * np.arange(1, RDF_BINS + 1)
    # ordered pairs (and each point with itself) within r; nextafter below r so
    # that the count is of distances strictly below each bin edge
    c = tree.count_neighbors(tree, np.nextafter(r, 0))
    return (np.asarray(c, dtype=np.float64) - len(pts)) / 2


def spectrum_rel(Eg, Eo):
    n = min(len(Eg), len(Eo))
    Eg, Eo = np.asarray(Eg[:n]), np.asarray(Eo[:n])
    sig = Eo > 1e-3 * Eo.max()
    return float(np.max(np.abs(Eg[sig] - Eo[sig]) / Eo[sig]))


@pytest.fixture(scope="module")
def capi():
    from tpm import build, capi

    build.build()
    return capi


@pytest.fixture(scope="module")
def reference(oracle_lib):
    """The oracle's state after 1, 10 and 20 steps, and its statistics,
    spectrum and RDF after 10 and 20."""
    p, s, tau = case()
    o = oracle_lib.Oracle(p, s.npart)
    o.load(s)
    o.set_tau(tau)
    o.initialize()
    snaps = {}
    for n in range(1, NSTEPS + 1):
        o.step()
        if n in (1, 10, 20):
            snap = {g: o.get_field(g) for g in FIELDS + ("Q",)}
            snap["part"] = o.get_particles(0)
            snap["rhs_t"] = o.get_rhs_t()
            snap["scalars"] = o.scalars()
            if n % 10 == 0:
                snap["stats"] = o.statistics()
                snap["E"] = oracle_lib.spectrum(p, snap["RU"], snap["RHO"])[0]
                snap["rdf"] = rdf_cumulative(p, snap["part"])
            snaps[n] = snap
    o.close()
    return snaps


def assert_close(ctx, snap, tol, p):
    for g in FIELDS:
        e = rel_err(ctx.download_field(g), snap[g])
        assert e <= tol, (g, e)
    assert rel_err(ctx.download_field("Q"), snap["Q"]) <= 10 * tol
    a = ctx.download_particles("base")
    b = snap["part"]
    assert np.array_equal(a["flag"], b["flag"])
    for q in inputs.PQ:
        e = rel_err(a[q], b[q])
        assert e <= tol, (q, e)
    assert abs(ctx.scalars()["P0"] - snap["scalars"]["P0"]) <= tol * abs(snap["scalars"]["P0"])
    return a


def assert_stats_close(ctx, snap, p):
    g, o = ctx.statistics(), snap["stats"]
    for k in ("TKE", "dissipation", "u_rms", "C_var", "Tg_mean", "Tp_mean"):
        assert abs(g[k] - o[k]) <= TOL_STATS * abs(o[k]), (k, g[k], o[k])
    E, _ = ctx.spectrum()
    assert spectrum_rel(E, snap["E"]) <= TOL_STATS
    pairs, _ = ctx.rdf(RDF_RMAX, RDF_BINS)
    cg = np.cumsum(pairs.astype(np.float64))
    co = snap["rdf"]
    assert np.all(np.abs(cg[2:] - co[2:]) <= TOL_STATS * co[2:]), (cg, co)


def gpu_context(capi, precision):
    p, s, tau = case(precision)
    ctx = capi.Context(p, s.npart)
    ctx.load(s)
    ctx.set_tau(tau)
    ctx.initialize()
    return p, ctx


def test_config1_fp64_matches_oracle_and_statistics(capi, reference):
    p, ctx = gpu_context(capi, P.PREC_FP64)
    ctx.run(1)
    ctx.sync()
    assert_close(ctx, reference[1], TOL1, p)
    ctx.run(9)
    ctx.sync()
    a = assert_close(ctx, reference[10], TOL10, p)
    b = reference[10]["part"]
    for q, L, n in (("x", p.Lx, p.Nx), ("y", p.Ly, p.Ny), ("z", p.Lz, p.Nz)):
        idx = 1.0 / (L / n)
        assert np.array_equal((a[q] * idx).astype(np.int64), (b[q] * idx).astype(np.int64)), q
        assert np.array_equal(np.round(a[q] * idx), np.round(b[q] * idx)), q
    assert_stats_close(ctx, reference[10], p)
    ctx.run(10)
    ctx.sync()
    assert_stats_close(ctx, reference[20], p)


def test_config1_mixed_matches_oracle_and_statistics(capi, reference):
    p, ctx = gpu_context(capi, P.PREC_MIXED)
    for n, more in ((1, 1), (10, 9)):
        ctx.run(more)
        ctx.sync()
        assert_close(ctx, reference[n], TOL_MIXED, p)
        assert ctx.scalars()["max_abs_div"] <= 1e-10
    assert_stats_close(ctx, reference[10], p)
    ctx.run(10)
    ctx.sync()
    assert_stats_close(ctx, reference[20], p)
