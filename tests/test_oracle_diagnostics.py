"""The oracle's diagnostics (CPU): grid::Statistics pinned to the reference's
own stat files, and the spectrum, dissipation and pair-count definitions
checked against identities that hold exactly on the staggered grid.
"""
import numpy as np
import pytest

from golden import STATS_NAMES, load
from tpm import inputs, params as P

# grid::Statistics writes with the default stream precision (6 significant
# digits): half a unit in the 6th digit relative to a leading digit of 1
TOL_PRINTED = 6e-6


@pytest.mark.parametrize("name", STATS_NAMES)
def test_oracle_statistics_match_reference_stat_files(oracle_lib, name):
    p, s, ref, nsteps, _ = load(name)
    o = oracle_lib.Oracle(p, s.npart)
    o.load(s)
    o.initialize()
    for st in range(nsteps):
        o.step()
        got = o.statistics()
        for key, vals in ref["stats"].items():
            r, g = float(vals[st]), got[key]
            assert abs(g - r) <= TOL_PRINTED * abs(r) + 1e-300, (st, key, g, r)


def test_oracle_statistics_before_the_first_step(oracle_lib):
    p = P.physical(16, 500, nu=0.02, A=0.1, tau_p=0.1, mass_loading=0.5, heating_Q=0.5)
    s = inputs.make_state(p, 500, seed=3)
    o = oracle_lib.Oracle(p, s.npart)
    o.load(s)
    o.initialize()
    st = o.statistics()
    assert st["TKE2"] == 0 and st["HT_mean"] == 0 and st["num_iteration"] == 0
    assert st["Rho_mean"] == 1.0 and st["Rho_min"] == 1.0 and st["P0"] == 1.0
    U = s.RU / p.Rho0
    assert abs(st["TKE"] - float(np.mean(U ** 2)) * 3) <= 1e-12 * st["TKE"]
    assert abs(st["u_rms"] - 1.0) <= 1e-12  # the generator scales u_rms to 1


def staggered_grad_sq(p, U):
    """sum_ij (D_j u_i)^2 with forward differences of the face values."""
    h = (p.Lx / p.Nx, p.Ly / p.Ny, p.Lz / p.Nz)
    tot = 0.0
    for i in range(3):
        for j, ax in enumerate((2, 1, 0)):
            tot += np.mean(((np.roll(U[i], -1, axis=ax) - U[i]) / h[j]) ** 2)
    return tot


@pytest.mark.parametrize("shape", [(16, 16, 16), (24, 16, 20)])
def test_dissipation_equals_half_gradient_norm_for_divergence_free_field(oracle_lib, shape):
    """On the periodic staggered grid the cross terms <D_j u_i D_i u_j> sum by
    parts to <(div u)^2> = 0, so <S:S> = <|grad u|^2>/2 exactly."""
    nx, ny, nz = shape
    p = P.physical(nx, 1, nu=0.02, A=0.1, tau_p=0.1, mass_loading=0.1)
    p = p.replace(Ny=ny, Nz=nz, Ly=p.Lx * ny / nx, Lz=p.Lx * nz / nx)
    U = inputs.solenoidal_velocity(p, seed=4)
    s = inputs.State(RU=U * p.Rho0, Rho=np.full((nz, ny, nx), p.Rho0), P=np.zeros((nz, ny, nx)),
                     part=inputs.random_particles(p, 1, 4), P0=p.P0)
    o = oracle_lib.Oracle(p, 1)
    o.load(s)
    o.initialize()
    st = o.statistics()
    nu = p.Mu0 / p.Rho0
    want = nu * staggered_grad_sq(p, U)
    assert abs(st["dissipation"] - want) <= 1e-12 * want


def test_spectrum_sums_to_kinetic_energy_and_matches_gradient_norm(oracle_lib):
    p = P.physical(24, 1, nu=0.02, A=0.1, tau_p=0.1, mass_loading=0.1)
    U = inputs.solenoidal_velocity(p, seed=5)
    Rho = 1.0 + 0.05 * np.random.default_rng(5).random((p.Nz, p.Ny, p.Nx))
    RU = U * 1.0
    E, dk = oracle_lib.spectrum(p, RU, Rho)
    Uf = oracle_lib.face_velocity(RU, Rho)
    assert abs(E.sum() - 0.5 * np.mean(Uf ** 2) * 3) <= 1e-13 * E.sum()
    assert dk == 1.0
    # shells: integer |k| rounded, the largest at about sqrt(3) N/2
    assert E.shape[0] == int(np.floor(np.sqrt(3) * 12 + 0.5)) + 1


def test_rdf_pairs_match_brute_force(oracle_lib):
    rng = np.random.default_rng(6)
    L = (2 * np.pi, 2 * np.pi, np.pi)
    n = 400
    x = rng.random(n) * L[0]
    y = rng.random(n) * L[1]
    z = rng.random(n) * L[2]
    x[:5] = 0.0
    x[5:10] = L[0]  # on the periodic boundary
    r_max, nb = 1.0, 20
    got = oracle_lib.rdf_pairs(x, y, z, L, r_max, nb)
    want = np.zeros(nb, dtype=np.uint64)
    for i in range(n):
        d = np.stack([x[i + 1:] - x[i], y[i + 1:] - y[i], z[i + 1:] - z[i]])
        for a in range(3):
            h = 0.5 * L[a]
            d[a] = np.where(d[a] > h, d[a] - L[a], np.where(d[a] < -h, d[a] + L[a], d[a]))
        r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2]
        r = np.sqrt(r2[r2 < r_max * r_max])
        b = (r / (r_max / nb)).astype(np.int64)
        np.add.at(want, b[b < nb], 1)
    assert np.array_equal(got, want)
