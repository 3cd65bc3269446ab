"""CPU REFERENCE GRADIENT - TEST INFRASTRUCTURE ONLY.

A NumPy restatement of the discrete adjoint of the RK4 step as the C oracle
(tpm_oracle.c) computes it, for the regime of the adjoint workload: no particle
heating (I0 = 0), no cooling, no gravity, uniform density.  There the density
stays uniform to the Poisson tolerance, so the step is the reference's
incompressible two-way-coupled update (simulation.cpp:60-91, grid.cpp:776-900,
particle.cpp:314-520) and its adjoint treats Rho_face, and with it the Poisson
coefficient, as the constants the forward run had.

Only tests/ import this module: it is the small-grid FP64 reference gradient
that the GPU adjoint (tpm_adjoint_run) is checked against, itself checked
against central finite differences of the oracle.

Objective (at the final step boundary):
    J = w_tke * 0.5 * sum_d mean(RU_d^2 / Rho_face_d) + w_cvar * var(C),
C the cloud-in-cell concentration of the final particle positions
(particle.cpp:522-555 weights), var = mean(C^2) - mean(C)^2 (tensor0.cpp:516-519).
Gradients: with respect to the initial momentum RU(0) (projected onto
discretely divergence-free fields, the admissible initial conditions), the
forcing coefficient A and a uniform Stokes time tau_p.
"""
from __future__ import annotations

import numpy as np

from tpm import inputs

PRE = (0.5, 0.5, 1.0, 1.0 / 6.0)     # grid.cpp:18-21
POST = (1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0)
AX = (2, 1, 0)  # array axis of the x, y, z direction ([Nz][Ny][Nx])


# ----------------------------------------------------------- grid operators
def sh(f, d, k):
    """f[i + k e_d] (periodic)."""
    return np.roll(f, -k, axis=AX[d])


def i_c2f(f, d):
    return (f + sh(f, d, -1)) * 0.5


def i_c2f_T(g, d):
    return (g + sh(g, d, 1)) * 0.5


def d_f2c(f, d, h):
    return (sh(f, d, 1) - f) / h[d]


def d_f2c_T(g, d, h):
    return (sh(g, d, -1) - g) / h[d]


def div_f2c(V, h):
    return sum(d_f2c(V[d], d, h) for d in range(3))


def grad_c2f(f, h):
    return np.stack([(f - sh(f, d, -1)) / h[d] for d in range(3)])


def del2(f, h):
    return sum((sh(f, d, 1) - 2 * f + sh(f, d, -1)) / h[d] ** 2 for d in range(3))


def lap_solve(f, p):
    """phi with div_f2c(grad_c2f(phi)) = f on the mean-free space (FFT)."""
    mwn = []
    for n, L, d in ((p.Nz, p.Lz, 0), (p.Ny, p.Ly, 1), (p.Nx, p.Lx, 2)):
        h = L / n
        k = np.fft.fftfreq(n, d=1.0 / n) * (2 * np.pi / L)
        mwn.append((2.0 / h ** 2) * (1 - np.cos(k * h)))
    tot = mwn[0][:, None, None] + mwn[1][None, :, None] + mwn[2][None, None, :]
    F = np.fft.fftn(f)
    tot[0, 0, 0] = 1.0
    F = -F / tot
    F[0, 0, 0] = 0.0
    return np.real(np.fft.ifftn(F))


def proj_T(lam_new, lam_np1, ratio, h, p):
    """lam_new - G Lap^-1 D (lam_new + ratio * lam_np1) (the projection's
    transpose with the np1 cross term; C = 1 for the uniform density)."""
    phi = lap_solve(div_f2c(lam_new + ratio * lam_np1, h), p)
    return lam_new - grad_c2f(phi, h)


# ------------------------------------------------------------- particles
def trunc_w(x, idx, n):
    """Truncation index and fraction of gas2part_velocity (particle.cpp:340-360)."""
    t = (x * idx).astype(np.int64)
    xl = x * idx - t
    return np.mod(t, n), xl


def interp(U, X, p):
    """(ug, vg, wg) at the particles, and the cell / fraction per direction."""
    idx = (p.Nx / p.Lx, p.Ny / p.Ly, p.Nz / p.Lz)
    n = (p.Nx, p.Ny, p.Nz)
    w = [trunc_w(X[d], idx[d], n[d]) for d in range(3)]
    i0, j0, k0 = w[0][0], w[1][0], w[2][0]
    g = []
    for d in range(3):
        lo = [i0, j0, k0]
        hi = list(lo)
        hi[d] = np.mod(lo[d] + 1, n[d])
        xl = w[d][1]
        g.append(xl * U[d][hi[2], hi[1], hi[0]] + (1 - xl) * U[d][lo[2], lo[1], lo[0]])
    return np.stack(g), w, idx, n


def cic_conc(X, p):
    """part2gas_concentration weights (particle.cpp:522-555) and C."""
    idx = (p.Nx / p.Lx, p.Ny / p.Ly, p.Nz / p.Lz)
    n = (p.Nx, p.Ny, p.Nz)
    r = [np.round(X[d] * idx[d]).astype(np.int64) for d in range(3)]  # half away from zero
    r = [np.where(np.abs(X[d] * idx[d] - np.trunc(X[d] * idx[d])) == 0.5,
                  np.trunc(X[d] * idx[d]) + np.sign(X[d]), r[d]).astype(np.int64) for d in range(3)]
    l = [X[d] * idx[d] - r[d] + 0.5 for d in range(3)]
    C = np.zeros((p.Nz, p.Ny, p.Nx))
    corners = []
    for a in (1, 0):
        for b in (1, 0):
            for c in (1, 0):
                ii = np.mod(r[0] - (1 - a), n[0])
                jj = np.mod(r[1] - (1 - b), n[1])
                kk = np.mod(r[2] - (1 - c), n[2])
                wx = l[0] if a else 1 - l[0]
                wy = l[1] if b else 1 - l[1]
                wz = l[2] if c else 1 - l[2]
                np.add.at(C, (kk, jj, ii), wx * wy * wz)
                corners.append((a, b, c, ii, jj, kk))
    return C, corners, l, idx


# --------------------------------------------------------------- forward
def record(o, p, nsteps):
    """Replays nsteps of the oracle stage by stage, keeping what the adjoint
    linearises about: RU_int, Rho_int, Rho_new and the int particle set."""
    traj = []
    for _ in range(nsteps):
        stages = []
        for s in range(4):
            part = o.get_particles(1)
            rec = dict(RU_int=o.get_field("RU_INT"), Rho_int=o.get_field("RHO_INT"),
                       X=np.stack([part[q] for q in ("x", "y", "z")]),
                       V=np.stack([part[q] for q in ("u", "v", "w")]))
            o.substep(s)
            rec["Rho_new"] = o.get_field("RHO_INT")
            stages.append(rec)
        o.end_step()
        traj.append(stages)
    return traj


def objective(p, RU, Rho, X, w_tke, w_cvar):
    rf = np.stack([i_c2f(Rho, d) for d in range(3)])
    n = p.Nx * p.Ny * p.Nz
    tke = 0.5 * float(np.sum(RU * RU / rf)) / n
    C, _, _, _ = cic_conc(X, p)
    var = float(np.mean(C * C) - np.mean(C) ** 2)
    return w_tke * tke + w_cvar * var


# --------------------------------------------------------------- adjoint
def rhs_adjoint(lam, RU, U, rf, p, A, h):
    """Adjoint of RHS = (mu/3) G D U + mu Lap U - conv(U, RU_int) + A RU_int
    (grid.cpp:776-814) w.r.t. RU_int (U = RU_int / Rho_face).  Returns
    (lam_RUint, <lam, RU_int>)."""
    mu = p.Mu0
    lamU = (mu / 3.0) * grad_c2f(div_f2c(lam, h), h) + mu * np.stack([del2(lam[d], h) for d in range(3)])
    lamRU = np.zeros_like(RU)
    # conv_d = sum_a D_a( I_a(U_d) * I_d(RU_a) ), entering the RHS with a minus
    for d in range(3):
        for a in range(3):
            m = d_f2c_T(-lam[d], a, h)
            lamU[d] += i_c2f_T(m * i_c2f(RU[a], d), a)
            lamRU[a] += i_c2f_T(m * i_c2f(U[d], a), d)
    return lamU / rf + lamRU + A * lam, float(np.sum(lam * RU))


def gradient(p, s0: inputs.State, nsteps, w_tke, w_cvar, oracle_lib, tau=None):
    """J and (dJ/dRU0 projected, dJ/dA, dJ/dtau) by the discrete adjoint."""
    o = oracle_lib.Oracle(p, s0.npart)
    o.load(s0)
    if tau is not None:
        o.set_tau(np.full(s0.npart, tau))
    o.initialize()
    traj = record(o, p, nsteps)
    RUf, Rhof = o.get_field("RU"), o.get_field("RHO")
    part = o.get_particles(0)
    Xf = np.stack([part[q] for q in ("x", "y", "z")])
    J = objective(p, RUf, Rhof, Xf, w_tke, w_cvar)
    h = (p.Lx / p.Nx, p.Ly / p.Ny, p.Lz / p.Nz)
    n = p.Nx * p.Ny * p.Nz
    npart = s0.npart
    tau_p = tau if tau is not None else p.Tp
    iTp = 1.0 / tau_p
    A = p.A1
    mpV = p.mp / (h[0] * h[1] * h[2])
    dt = p.dt
    # ---- dJ/d(final state)
    rf = np.stack([i_c2f(Rhof, d) for d in range(3)])
    lam_RU = w_tke * RUf / rf / n
    lam_RUint0 = np.zeros_like(RUf)
    C, corners, l, idx = cic_conc(Xf, p)
    dC = w_cvar * (2.0 * C / n - 2.0 * C.mean() / n)
    lam_X = np.zeros((3, npart))
    for a, b, c, ii, jj, kk in corners:
        g = dC[kk, jj, ii]
        wx = l[0] if a else 1 - l[0]
        wy = l[1] if b else 1 - l[1]
        wz = l[2] if c else 1 - l[2]
        sx, sy, sz = (1 if a else -1), (1 if b else -1), (1 if c else -1)
        lam_X[0] += g * sx * idx[0] * wy * wz
        lam_X[1] += g * wx * sy * idx[1] * wz
        lam_X[2] += g * wx * wy * sz * idx[2]
    lam_V = np.zeros((3, npart))
    lam_Xint0 = np.zeros((3, npart))
    lam_Vint0 = np.zeros((3, npart))
    gA = 0.0
    gtau = 0.0
    for stages in reversed(traj):
        # end of step: RU_next = RU_np1 - mean (make_mean_U0), RU_int0_next = RU_np1,
        # particles: base_next = int0_next = np1
        lam_np1 = lam_RU - lam_RU.mean(axis=(1, 2, 3), keepdims=True) + lam_RUint0
        lam_Xnp1 = lam_X + lam_Xint0
        lam_Vnp1 = lam_V + lam_Vint0
        lam_new = np.zeros_like(lam_np1)
        lam_Xnew = np.zeros_like(lam_X)
        lam_Vnew = np.zeros_like(lam_V)
        lam_RUb = np.zeros_like(lam_np1)
        lam_Xb = np.zeros_like(lam_X)
        lam_Vb = np.zeros_like(lam_V)
        for s in (3, 2, 1, 0):
            rec = stages[s]
            a, b = dt * PRE[s], dt * POST[s]
            if s == 3:  # RU_new = RU_np1 (aliases), projected together
                lam_np1 = proj_T(lam_np1, 0 * lam_np1, 0.0, h, p)
                lam_RHS = b * lam_np1
                lam_Vint = b * lam_Xnp1
                lam_RHSu = b * lam_Vnp1
            else:
                lam_newp = proj_T(lam_new, lam_np1, b / a, h, p)
                lam_RHS = b * lam_np1 + a * lam_newp
                lam_RUb += lam_newp
                lam_Xb += lam_Xnew
                lam_Vint = a * lam_Xnew + b * lam_Xnp1
                lam_Vb += lam_Vnew
                lam_RHSu = a * lam_Vnew + b * lam_Vnp1
            RU = rec["RU_int"]
            rfs = np.stack([i_c2f(rec["Rho_int"], d) for d in range(3)])
            U = RU / rfs
            X, V = rec["X"], rec["V"]
            ug, w, pidx, pn = interp(U, X, p)
            RHSu = (ug - V) * iTp
            lam_Xint = np.zeros_like(X)
            # two-way force: RHS += -(mp/Vcell) F_p, F_p = deposit(RHSu at x_int)
            lam_F = -mpV * lam_RHS if p.TWC else np.zeros_like(lam_RHS)
            i0, j0, k0 = w[0][0], w[1][0], w[2][0]
            lamU = np.zeros_like(U)
            for d in range(3):
                lo = [i0, j0, k0]
                hi = list(lo)
                hi[d] = np.mod(lo[d] + 1, pn[d])
                xl = w[d][1]
                Fhi, Flo = lam_F[d][hi[2], hi[1], hi[0]], lam_F[d][lo[2], lo[1], lo[0]]
                lam_RHSu[d] += xl * Fhi + (1 - xl) * Flo
                lam_Xint[d] += RHSu[d] * pidx[d] * (Fhi - Flo)
            # RHSu = (ug - u_int) / tau
            lam_ug = iTp * lam_RHSu
            lam_Vint = lam_Vint - iTp * lam_RHSu
            gtau += float(np.sum(lam_RHSu * (-(ug - V) / tau_p ** 2)))
            for d in range(3):
                lo = [i0, j0, k0]
                hi = list(lo)
                hi[d] = np.mod(lo[d] + 1, pn[d])
                xl = w[d][1]
                np.add.at(lamU[d], (hi[2], hi[1], hi[0]), xl * lam_ug[d])
                np.add.at(lamU[d], (lo[2], lo[1], lo[0]), (1 - xl) * lam_ug[d])
                Uhi, Ulo = U[d][hi[2], hi[1], hi[0]], U[d][lo[2], lo[1], lo[0]]
                lam_Xint[d] += lam_ug[d] * pidx[d] * (Uhi - Ulo)
            lam_RUint, gA_s = rhs_adjoint(lam_RHS, RU, U, rfs, p, A, h)
            lam_RUint += lamU / rfs
            gA += gA_s
            lam_new, lam_Xnew, lam_Vnew = lam_RUint, lam_Xint, lam_Vint
        # stage 0's int inputs are this step's RU_int0 / particle int0; its np1
        # inputs are the base state
        lam_RUint0 = lam_new
        lam_RU = lam_RUb + lam_np1
        lam_Xint0, lam_Vint0 = lam_Xnew, lam_Vnew
        lam_X = lam_Xb + lam_Xnp1
        lam_V = lam_Vb + lam_Vnp1
    gRU = lam_RU + lam_RUint0  # at t = 0, RU_int = RU (grid.cpp:461-472)
    gRU = proj_T(gRU, 0 * gRU, 0.0, h, p)
    return J, gRU, gA, gtau


def forward_J(p, s0: inputs.State, nsteps, w_tke, w_cvar, oracle_lib, tau=None):
    o = oracle_lib.Oracle(p, s0.npart)
    o.load(s0)
    if tau is not None:
        o.set_tau(np.full(s0.npart, tau))
    o.initialize()
    for _ in range(nsteps):
        for s in range(4):
            o.substep(s)
        o.end_step()
    part = o.get_particles(0)
    X = np.stack([part[q] for q in ("x", "y", "z")])
    return objective(p, o.get_field("RU"), o.get_field("RHO"), X, w_tke, w_cvar)
