"""The reference-shaped boundary above the C ABI: the reference's time loop
(simulation.cpp:57-93) written in C++ against the grid facade
(include/tpm_grid.hpp) and linked with g++ against libtpm.so
(tests/simulation_loop.cpp), and the per-method entry points behind it
(tpm_update_rho ... tpm_time_advance).

CPU: the program compiles and links.  GPU: it reproduces the golden fixture
made by the reference's own build (heated, two-way coupled 16^3 box, 2 steps)
to 1e-12; the per-method calls give the same bits as the fused step; calls
out of the reference's order are refused without queuing work.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import REPO, rel_err

HERE = os.path.dirname(os.path.abspath(__file__))
TOL = 1e-12


def compile_loop(out_dir):
    from tpm import build

    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    lib = build.build()
    libdir = os.path.dirname(lib)
    exe = os.path.join(str(out_dir), "simulation_loop")
    subprocess.check_call([gxx, "-O2", "-std=c++17", "-I", os.path.join(REPO, "include"),
                           os.path.join(HERE, "simulation_loop.cpp"), "-o", exe,
                           "-L", libdir, "-ltpm", f"-Wl,-rpath,{libdir}"])
    return exe


def test_cpp_loop_compiles_and_links(tmp_path):
    exe = compile_loop(tmp_path)
    assert os.access(exe, os.X_OK)


@pytest.mark.gpu
def test_cpp_loop_matches_reference_golden(tmp_path):
    from golden import load
    from tpm import inputs

    exe = compile_loop(tmp_path)
    p, s, ref, nsteps, _ = load("heated16_2steps")
    src, out = tmp_path / "in", tmp_path / "out"
    inputs.write_restart(str(src), p, s)
    (tmp_path / "params.bin").write_bytes(bytes(p.to_c()))
    os.makedirs(out)
    env = dict(os.environ)
    cuda_lib = os.path.join(os.path.dirname(os.path.dirname(shutil.which("nvcc") or
                                                            "/usr/local/cuda/bin/nvcc")), "lib64")
    env["LD_LIBRARY_PATH"] = cuda_lib + os.pathsep + env.get("LD_LIBRARY_PATH", "")
    r = subprocess.run([exe, str(tmp_path / "params.bin"), str(s.npart), str(src), str(nsteps),
                        str(out)], capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = r.stdout.strip().splitlines()
    assert len(lines) == nsteps and lines[-1].startswith(f"step {nsteps} ")
    got = inputs.read_restart(str(out), p)
    for name, a, b in (("RU", got.RU, ref["RU"]), ("Rho", got.Rho, ref["Rho"]),
                       ("P", got.P, ref["P"])):
        e = rel_err(a, b)
        assert e <= TOL, (name, e)
    assert np.array_equal(got.part["flag"], ref["part"]["flag"])
    for q in inputs.PQ:
        assert rel_err(got.part[q], ref["part"][q]) <= TOL, q
    assert abs(got.P0 - ref["P0"]) <= 1e-13 * abs(ref["P0"])
    assert got.num_timestep == nsteps


def phase_step(ctx):
    """One step through the per-method entry points, in simulation.cpp's order."""
    L, h = ctx.L, ctx.h
    ctx._check(L.tpm_param_update(h))
    for k in range(4):
        for fn in (L.tpm_update_rho, L.tpm_update_p0, L.tpm_update_particle):
            ctx._check(fn(h, k))
        if ctx.p.solve_for_scalar:
            ctx._check(L.tpm_update_passive_scalar(h, k))
        for fn in (L.tpm_update_ru_wop, L.tpm_compute_div_u_new, L.tpm_compute_rhs_pois,
                   L.tpm_solve_poisson, L.tpm_update_ru_wp, L.tpm_time_advance_rk4):
            ctx._check(fn(h, k))
    ctx._check(L.tpm_make_mean_u0(h))
    ctx._check(L.tpm_time_advance(h))


@pytest.mark.gpu
@pytest.mark.parametrize("precision,n", [("fp64", 24), ("mixed", 24), ("mixed", 32)])
def test_method_calls_equal_the_fused_step(precision, n):
    """Two steps by the per-method entry points are bit-identical to two
    fused steps, on both paths (heated, two-way coupled, passive scalar on);
    at 32^3 the mixed path's density pass also forms the face velocity and its
    Poisson right-hand-side pass the face coefficients (TMA-fed tiles)."""
    from tpm import build, capi, inputs, params as P

    build.build()
    prec = P.PREC_MIXED if precision == "mixed" else P.PREC_FP64
    p = P.physical(n, 3000, nu=0.02, A=0.1, tau_p=0.1, mass_loading=0.5, heating_Q=0.5,
                   iterations=20, epsilon=1e-13, precision=prec)
    s = inputs.make_state(p, 3000, seed=14)
    s.PS = inputs.passive_scalar(p, seed=14)
    p = p.replace(dt=inputs.cfl_dt(p, s.RU), solve_for_scalar=1, D_M=0.01)
    out = []
    for how in ("fused", "methods"):
        ctx = capi.Context(p, s.npart)
        ctx.load(s)
        ctx.initialize()
        for _ in range(2):
            if how == "fused":
                ctx.step()
            else:
                phase_step(ctx)
        ctx.sync()
        out.append(ctx)
    a, b = out
    for g in ("RU", "RU_INT", "RHO", "P", "C", "Q", "PASSIVE_SCALAR"):
        assert np.array_equal(a.download_field(g), b.download_field(g)), g
    pa, pb = a.download_particles("base"), b.download_particles("base")
    for q in inputs.PQ:
        assert np.array_equal(pa[q], pb[q]), q
    sa, sb = a.scalars(), b.scalars()
    assert sa["P0"] == sb["P0"] and sa["T_cur"] == sb["T_cur"]
    assert sa["num_timestep"] == sb["num_timestep"] == 2


@pytest.mark.gpu
def test_method_calls_out_of_order_are_refused():
    from tpm import build, capi, inputs, params as P

    build.build()
    p = P.physical(16, 500, nu=0.02, A=0.1, tau_p=0.1, mass_loading=0.5, heating_Q=0.5)
    s = inputs.make_state(p, 500, seed=3)
    p = p.replace(dt=inputs.cfl_dt(p, s.RU))
    ctx = capi.Context(p, s.npart)
    L, h = ctx.L, ctx.h
    assert L.tpm_update_rho(h, 0) == -6  # before tpm_initialize
    ctx.load(s)
    ctx.initialize()
    P0 = ctx.download_field("P")
    STATE = -6
    assert L.tpm_solve_poisson(h, 0) == STATE       # projection before the density update
    assert L.tpm_update_rho(h, 1) == STATE          # wrong stage
    assert L.tpm_make_mean_u0(h) == STATE           # before the fourth stage
    assert L.tpm_time_advance(h) == STATE
    assert L.tpm_update_passive_scalar(h, 0) == STATE  # solve_for_scalar off
    assert L.tpm_update_rho(h, 0) == 0
    assert L.tpm_update_rho(h, 0) == STATE          # twice
    assert L.tpm_update_p0(h, 0) == 0               # queued by Update_Rho already: no-op
    assert L.tpm_update_p0(h, 0) == STATE
    assert L.tpm_compute_rhs_pois(h, 0) == STATE    # Compute_Div_U_new not yet
    assert L.tpm_substep(h, 0) == STATE             # a stage is in progress
    assert L.tpm_step(h) == STATE
    ctx.sync()
    assert np.array_equal(ctx.download_field("P"), P0)  # nothing projected
