"""Run parameters: ctypes mirror of ``tpm_params`` (include/tpm.h) plus the
reference's positional parameter deck (params.cpp:23-63) and the derived
constants params.cpp:70-77 computes.

The deck writer lets the GPU library, the C oracle and the reference's own
build run from one configuration: every double is written with 17 significant
digits so the reference's ``istream >> double`` reads back the same value.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field, fields

PI = 3.141592653589793  # params.h:5
PREC_FP64 = 0
PREC_MIXED = 1


class TpmParams(ctypes.Structure):
    """Binary layout of ``struct tpm_params`` in include/tpm.h."""

    _fields_ = [
        ("Nx", ctypes.c_int32), ("Ny", ctypes.c_int32), ("Nz", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("Lx", ctypes.c_double), ("Ly", ctypes.c_double), ("Lz", ctypes.c_double),
        ("dt", ctypes.c_double), ("threshold", ctypes.c_double),
        ("cooling", ctypes.c_int32), ("Iteration1", ctypes.c_int32),
        ("Iteration2", ctypes.c_int32), ("TWC", ctypes.c_int32),
        ("epsilon", ctypes.c_double),
        ("ParticleGravity", ctypes.c_int32), ("elongated_box", ctypes.c_int32),
        ("solve_for_scalar", ctypes.c_int32), ("solve_for_vector", ctypes.c_int32),
        ("A1", ctypes.c_double), ("A2", ctypes.c_double), ("Rho0", ctypes.c_double),
        ("U0", ctypes.c_double), ("V0", ctypes.c_double), ("W0", ctypes.c_double),
        ("T0", ctypes.c_double), ("Mu0", ctypes.c_double), ("k", ctypes.c_double),
        ("gx1", ctypes.c_double), ("gy1", ctypes.c_double), ("gz1", ctypes.c_double),
        ("gx2", ctypes.c_double), ("gy2", ctypes.c_double), ("gz2", ctypes.c_double),
        ("Cp", ctypes.c_double), ("Cv", ctypes.c_double), ("np0", ctypes.c_double),
        ("Dp", ctypes.c_double), ("Rhop", ctypes.c_double), ("Cvp", ctypes.c_double),
        ("epsilonp", ctypes.c_double), ("Nu", ctypes.c_double),
        ("I01", ctypes.c_double), ("I02", ctypes.c_double),
        ("D_M", ctypes.c_double), ("S1_type", ctypes.c_int32), ("Solver", ctypes.c_int32),
    ]


class TpmScalars(ctypes.Structure):
    """Binary layout of ``struct tpm_scalars`` in include/tpm.h."""

    _fields_ = [
        ("P0", ctypes.c_double), ("P0_int", ctypes.c_double),
        ("P0_new", ctypes.c_double), ("P0_np1", ctypes.c_double),
        ("T_cur", ctypes.c_double), ("num_timestep", ctypes.c_int64),
        ("last_poisson_iterations", ctypes.c_int32),
        ("total_poisson_iterations", ctypes.c_int32),
        ("last_poisson_error", ctypes.c_double), ("max_abs_div", ctypes.c_double),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class TpmStats(ctypes.Structure):
    """Binary layout of ``struct tpm_stats`` in include/tpm.h."""

    _fields_ = [("T_cur", ctypes.c_double), ("num_timestep", ctypes.c_int64)] + [
        (n, ctypes.c_double) for n in (
            "Rho_mean", "Rho_max", "Rho_min", "C_mean", "C_max", "C_min", "TKE2",
            "TKE_U", "TKE_V", "TKE_W", "TKE", "Gas_CFL_Max", "Gas_Max_Diff_CFL", "u_max",
            "Vp_max", "Tp_max", "Tp_mean", "HT_mean", "Tg_mean", "P0")
    ] + [("num_iteration", ctypes.c_int32), ("reserved", ctypes.c_int32)] + [
        (n, ctypes.c_double) for n in ("C_var", "u_rms", "dissipation", "Passive_Scalar_mean")
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_ if name != "reserved"}


@dataclass
class Params:
    """The deck fields the substep uses (params.h:9-59), with reference names."""

    Nx: int = 32
    Ny: int = 32
    Nz: int = 32
    Lx: float = 2 * PI
    Ly: float = 2 * PI
    Lz: float = 2 * PI
    dt: float = 1e-3
    threshold: float = 1e30
    cooling: int = 0
    Iteration1: int = 20
    Iteration2: int = 20
    epsilon: float = 1e-13
    TWC: int = 1
    ParticleGravity: int = 0
    A1: float = 0.0
    A2: float = 0.0
    Rho0: float = 1.0
    U0: float = 0.0
    V0: float = 0.0
    W0: float = 0.0
    T0: float = 1.0
    Mu0: float = 0.01
    k: float = 0.05
    gx1: float = 0.0
    gy1: float = 0.0
    gz1: float = 0.0
    gx2: float = 0.0
    gy2: float = 0.0
    gz2: float = 0.0
    Cp: float = 3.5
    Cv: float = 2.5
    np0: float = 0.0
    Dp: float = 1e-3
    Rhop: float = 1e3
    Cvp: float = 2.5
    epsilonp: float = 1.0
    Nu: float = 2.0
    I01: float = 0.0
    I02: float = 0.0
    precision: int = PREC_FP64
    elongated_box: int = 0
    solve_for_scalar: int = 0
    solve_for_vector: int = 0
    D_M: float = 0.0          # passive-scalar diffusivity (params.h:51)
    S1_type: int = 1          # passive-scalar source type (params.h:53, token s1t)
    Solver: int = 0           # 0: FFT-preconditioned Richardson; 2: PCG (tpm_params.Solver)

    # ---- derived (params.cpp:70-77, params.h:133-138) ----
    @property
    def R(self) -> float:
        return self.Cp - self.Cv

    @property
    def P0(self) -> float:
        return self.Rho0 * self.T0 * self.R

    @property
    def Tp(self) -> float:
        return self.Rhop * self.Dp * self.Dp / (18 * self.Mu0)

    @property
    def mp(self) -> float:
        return self.Rhop * PI * self.Dp * self.Dp * self.Dp / 6.0

    @property
    def Vol(self) -> float:
        return self.Lx * self.Ly * self.Lz

    @property
    def N0(self) -> int:
        return int(self.np0 * self.Vol)

    @property
    def ncell(self) -> int:
        return self.Nx * self.Ny * self.Nz

    @property
    def dx(self) -> float:
        return self.Lx / self.Nx

    def to_c(self) -> TpmParams:
        c = TpmParams()
        for f in TpmParams._fields_:
            setattr(c, f[0], getattr(self, f[0]))
        return c

    def replace(self, **kw) -> "Params":
        d = {f.name: getattr(self, f.name) for f in fields(self)}
        d.update(kw)
        return Params(**d)

    # ---- reference deck (params.cpp:23-63) ----
    def deck_text(self, statistics: bool = False) -> str:
        g = lambda v: repr(float(v))  # shortest round-trip repr == %.17g semantics
        lines = [
            "# deck written by tpm.params (token order of params.cpp:23-63)",
            f"{self.Nx} {self.Ny} {self.Nz}",
            f"{g(self.Lx)} {g(self.Ly)} {g(self.Lz)}",
            f"{self.elongated_box}",
            f"{self.solve_for_scalar}",
            f"{self.solve_for_vector}",
            "1",  # bs
            "0",  # Np_track
            f"{g(1e30)} {g(self.dt)} {g(self.threshold)}",  # T_final dt threshold
            "1 0" if statistics else "0 0",  # Statistics Stat_print
            "1000000000 1000000000",  # Data_freq_fast Data_freq_slow
            "./ ./",  # Data_dir Stat_dir
            "1",  # Initial: restart files
            "1" if self.solve_for_scalar else "5",  # Initial_C: Restart_Passive_Scalar.bin
            "2",  # Initial_V: RV = 0
            f"0 {self.Solver}",  # PreCond Solver (0 = FFT)
            f"{self.cooling}",
            f"{self.Iteration1} {self.Iteration2} {g(self.epsilon)}",
            f"{self.TWC} {self.ParticleGravity}",
            f"{g(self.A1)} {g(self.A2)}",
            f"{g(self.Rho0)}",
            "1.0",  # Rho_forV
            f"{g(self.U0)} {g(self.V0)} {g(self.W0)}",
            "0 0 0",  # V0_1 V0_2 V0_3
            f"{g(self.T0)}",
            f"{g(self.Mu0)} {g(self.k)}",
            f"{g(self.gx1)} {g(self.gy1)} {g(self.gz1)} {g(self.gx2)} {g(self.gy2)} {g(self.gz2)}",
            f"{g(self.Cp)} {g(self.Cv)}",
            f"{g(self.np0)}",
            f"{g(self.Dp)} {g(self.Rhop)}",
            f"{g(self.Cvp)}",
            f"{g(self.epsilonp)}",
            f"{g(self.Nu)}",
            f"{g(self.I01)} {g(self.I02)}",
            f"{g(self.D_M)}",  # D_M
            "0",  # eta
            f"{self.S1_type}",  # s1t
            "1",  # s2t
        ]
        return "\n".join(lines) + "\n"


def np0_for(npart: int, vol: float) -> float:
    """Number density whose truncation (int)(np0*Vol) (params.h:129) is npart."""
    np0 = (npart + 0.5) / vol
    assert int(np0 * vol) == npart, (npart, np0, vol)
    return np0


def physical(N: int, npart: int, nu: float, A: float, tau_p: float, mass_loading: float,
             heating_Q: float = 0.0, dt: float = 1e-3, iterations: int = 20,
             epsilon: float = 1e-13, precision: int = PREC_FP64) -> Params:
    """Map a physical configuration onto deck parameters.

    L = 2*pi, Rho0 = T0 = 1, Cp = 3.5, Cv = 2.5 (R = 1, P0 = 1), Mu0 = nu*Rho0,
    k = Mu0*Cp/0.7 (Pr = 0.7).  Given the Stokes time tau_p and mass loading phi:
    mp = phi*Rho0*L^3/Np, Dp = mp/(3*pi*Mu0*tau_p), Rhop = 18*Mu0*tau_p/Dp^2, so
    that params.cpp:76-77 recover Tp = tau_p and mp.  A particle heating rate Q
    (temperature rise per unit time) sets I0 = Q*mp*Cvp/(0.25*eps_p*pi*Dp^2).
    """
    L = 2 * PI
    Rho0, Cp, Cv = 1.0, 3.5, 2.5
    Mu0 = nu * Rho0
    vol = L * L * L
    mp = mass_loading * Rho0 * vol / npart if npart > 0 else 1e-12
    Dp = mp / (3 * PI * Mu0 * tau_p)
    Rhop = 18 * Mu0 * tau_p / (Dp * Dp)
    Cvp, epsp = Cv, 1.0
    I0 = heating_Q * mp * Cvp / (0.25 * epsp * PI * Dp * Dp)
    return Params(
        Nx=N, Ny=N, Nz=N, Lx=L, Ly=L, Lz=L, dt=dt, Iteration1=iterations,
        Iteration2=iterations, epsilon=epsilon, TWC=1, A1=A, A2=A, Rho0=Rho0,
        T0=1.0, Mu0=Mu0, k=Mu0 * Cp / 0.7, Cp=Cp, Cv=Cv,
        np0=np0_for(npart, vol) if npart > 0 else 0.0, Dp=Dp, Rhop=Rhop, Cvp=Cvp,
        epsilonp=epsp, Nu=2.0, I01=I0, I02=I0, precision=precision)


# The five workloads of the benchmark suite (grid, particles, physics).
WORKLOADS = {
    "box32_p1e4": dict(N=32, npart=10_000, nu=0.02, A=0.1, tau_p=0.1, mass_loading=0.2,
                       heating_Q=0.0, seed=0),
    "box128_p1e6_heated": dict(N=128, npart=1_000_000, nu=0.005, A=0.1, tau_p=0.1,
                               mass_loading=0.5, heating_Q=0.1, seed=1),
    "box256_p8e6_heated": dict(N=256, npart=8_000_000, nu=0.002, A=0.1, tau_p=0.2,
                               mass_loading=1.0, heating_Q=0.1, seed=2),
    "box64_p2e5": dict(N=64, npart=200_000, nu=0.01, A=0.1, tau_p=0.1, mass_loading=0.3,
                       heating_Q=0.0, seed=3),
}


def ensemble_boxes(nboxes: int = 48, precision: int = PREC_MIXED):
    """The batched-ensemble workload: box b (seed b) has N drawn uniformly from
    {32, 48, 64, 96} and a particle count log-uniform in [1e4, 5e5], with the
    physics of the 32^3 workload (A = 0.1, tau_p = 0.1, mass loading 0.2, no
    heating) and nu set so that kmax*eta = 1.5.  With the seeded spectrum
    E(k) ~ k^4 exp(-2 (k/4)^2) at u_rms = 1, <|grad u|^2> = 2*(3/2)*20 = 60, so
    eps = 60 nu, eta = (nu^3/eps)^(1/4), and kmax = N/2 gives nu = sqrt(60)*9/N^2.
    Returns [(Params, npart, seed)]."""
    import numpy as np

    out = []
    for b in range(nboxes):
        rng = np.random.Generator(np.random.PCG64(b))
        N = int(rng.choice([32, 48, 64, 96]))
        npart = int(round(np.exp(rng.uniform(np.log(1e4), np.log(5e5)))))
        nu = float(np.sqrt(60.0) * 9.0 / N ** 2)
        p = physical(N, npart, nu=nu, A=0.1, tau_p=0.1, mass_loading=0.2, heating_Q=0.0,
                     iterations=20, epsilon=1e-13, precision=precision)
        out.append((p, npart, b))
    return out
