"""Seeded synthetic inputs and the reference's restart/dump byte formats.

* Velocity: Gaussian random Fourier modes with E(k) ~ k^4 exp(-2 (k/4)^2),
  projected onto the null space of the staggered-grid divergence
  (tensor0::Equal_Div_F2C, tensor0.cpp:249-256) so that div_F2C(u) = 0 to
  roundoff, zero mean, scaled to u_rms = 1 (mean(u^2+v^2+w^2)/3 = 1).
* Particles: uniform positions in [0, L)^3, zero velocity, T = T0, flag = id.
* Files: the formats the reference's Initial=1 branch reads (grid.cpp:221-238,
  particle.cpp:939-989): raw native FP64 fields in C order [Nz][Ny][Nx] with a
  vector field as its x, y, z blocks; particle quantities as FP64 [Np] and
  the flag as int32 [Np]; Restart_numbers.dat holds "P0 T_cur num_timestep".
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field

import numpy as np

from .params import Params

PQ = ("x", "y", "z", "u", "v", "w", "T")


@dataclass
class State:
    RU: np.ndarray            # (3, Nz, Ny, Nx)
    Rho: np.ndarray           # (Nz, Ny, Nx)
    P: np.ndarray             # (Nz, Ny, Nx)
    part: dict                # x,y,z,u,v,w,T float64 [Np]; flag int32 [Np]
    P0: float = 1.0
    T_cur: float = 0.0
    num_timestep: int = 0
    tau: np.ndarray | None = None   # optional per-particle Stokes time (extension)
    PS: np.ndarray | None = None    # optional passive scalar (Nz, Ny, Nx)

    @property
    def npart(self) -> int:
        return int(self.part["x"].shape[0])


def solenoidal_velocity(p: Params, seed: int, kpeak: float = 4.0) -> np.ndarray:
    """Random staggered velocity (3, Nz, Ny, Nx), discretely divergence-free."""
    rng = np.random.Generator(np.random.PCG64(seed))
    shape = (p.Nz, p.Ny, p.Nx)
    kz = np.fft.fftfreq(p.Nz, d=1.0 / p.Nz) * (2 * np.pi / p.Lz)
    ky = np.fft.fftfreq(p.Ny, d=1.0 / p.Ny) * (2 * np.pi / p.Ly)
    kx = np.fft.fftfreq(p.Nx, d=1.0 / p.Nx) * (2 * np.pi / p.Lx)
    KZ, KY, KX = np.meshgrid(kz, ky, kx, indexing="ij")
    kmag = np.sqrt(KX ** 2 + KY ** 2 + KZ ** 2)
    # amplitude per mode ~ sqrt(E(k) / (4 pi k^2)) with E ~ k^4 exp(-2 (k/k0)^2)
    amp = np.where(kmag > 0, kmag * np.exp(-(kmag / kpeak) ** 2), 0.0)
    uh = []
    for _ in range(3):
        w = rng.standard_normal(shape)
        uh.append(np.fft.fftn(w) * amp)
    # discrete divergence symbol of the face->centre difference (index shifts)
    ex = np.exp(2j * np.pi * np.fft.fftfreq(p.Nx))[None, None, :]
    ey = np.exp(2j * np.pi * np.fft.fftfreq(p.Ny))[None, :, None]
    ez = np.exp(2j * np.pi * np.fft.fftfreq(p.Nz))[:, None, None]
    D = [(ex - 1) / p.dx * np.ones(shape), (ey - 1) / (p.Ly / p.Ny) * np.ones(shape),
         (ez - 1) / (p.Lz / p.Nz) * np.ones(shape)]
    dd = sum(np.abs(d) ** 2 for d in D)
    dd[0, 0, 0] = 1.0
    div = sum(d * u for d, u in zip(D, uh))
    uh = [u - np.conj(d) * div / dd for d, u in zip(D, uh)]
    for u in uh:
        u[0, 0, 0] = 0.0
    U = np.stack([np.real(np.fft.ifftn(u)) for u in uh])
    urms = np.sqrt(np.mean(U[0] ** 2 + U[1] ** 2 + U[2] ** 2) / 3.0)
    return np.ascontiguousarray(U / urms)


def div_f2c(p: Params, U: np.ndarray) -> np.ndarray:
    """Staggered divergence (index shifts with periodic wrap)."""
    return ((np.roll(U[0], -1, axis=2) - U[0]) * (1.0 / (p.Lx / p.Nx))
            + (np.roll(U[1], -1, axis=1) - U[1]) * (1.0 / (p.Ly / p.Ny))
            + (np.roll(U[2], -1, axis=0) - U[2]) * (1.0 / (p.Lz / p.Nz)))


def cfl_dt(p: Params, U: np.ndarray, cfl: float = 0.3) -> float:
    """Fixed dt = cfl * dx / max|u0| (the reference has no adaptive dt)."""
    return float(cfl * p.dx / np.abs(U).max())


def random_particles(p: Params, npart: int, seed: int) -> dict:
    rng = np.random.Generator(np.random.PCG64(seed + 1_000_003))
    pos = rng.random((3, npart))
    part = {
        "x": pos[0] * p.Lx, "y": pos[1] * p.Ly, "z": pos[2] * p.Lz,
        "u": np.zeros(npart), "v": np.zeros(npart), "w": np.zeros(npart),
        "T": np.full(npart, p.T0),
        "flag": np.arange(npart, dtype=np.int32),
    }
    return part


def log_uniform_tau(npart: int, lo: float, hi: float, seed: int) -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(seed + 7))
    return np.exp(rng.uniform(np.log(lo), np.log(hi), npart))


def make_state(p: Params, npart: int, seed: int) -> State:
    U = solenoidal_velocity(p, seed)
    shape = (p.Nz, p.Ny, p.Nx)
    return State(RU=U * p.Rho0, Rho=np.full(shape, p.Rho0), P=np.zeros(shape),
                 part=random_particles(p, npart, seed), P0=p.P0, T_cur=0.0,
                 num_timestep=0)


# ------------------------------------------------------------------ files
def write_restart(dirpath: str, p: Params, s: State, statistics: bool = False) -> None:
    """Write deck + Restart_* files for the reference's Initial=1 branch."""
    os.makedirs(dirpath, exist_ok=True)
    with open(os.path.join(dirpath, "deck.txt"), "w") as f:
        f.write(p.deck_text(statistics))
    np.ascontiguousarray(s.RU, dtype=np.float64).tofile(os.path.join(dirpath, "Restart_RU.bin"))
    np.ascontiguousarray(s.Rho, dtype=np.float64).tofile(os.path.join(dirpath, "Restart_Rho.bin"))
    np.ascontiguousarray(s.P, dtype=np.float64).tofile(os.path.join(dirpath, "Restart_P.bin"))
    for q in PQ:
        np.ascontiguousarray(s.part[q], dtype=np.float64).tofile(
            os.path.join(dirpath, f"Restart_Part_{q}.bin"))
    np.ascontiguousarray(s.part["flag"], dtype=np.int32).tofile(
        os.path.join(dirpath, "Restart_Part_flag.bin"))
    with open(os.path.join(dirpath, "Restart_numbers.dat"), "w") as f:
        f.write(f"{s.P0!r} {s.T_cur!r} {s.num_timestep}\n")
    if s.PS is not None:  # read when Initial_C = 1 (grid.cpp:445-450)
        np.ascontiguousarray(s.PS, dtype=np.float64).tofile(
            os.path.join(dirpath, "Restart_Passive_Scalar.bin"))


def read_restart(dirpath: str, p: Params) -> State:
    shape = (p.Nz, p.Ny, p.Nx)
    rd = lambda n, dt=np.float64: np.fromfile(os.path.join(dirpath, n), dtype=dt)
    RU = rd("Restart_RU.bin").reshape((3,) + shape)
    part = {q: rd(f"Restart_Part_{q}.bin") for q in PQ}
    part["flag"] = rd("Restart_Part_flag.bin", np.int32)
    with open(os.path.join(dirpath, "Restart_numbers.dat")) as f:
        tok = f.read().split()
    ps = os.path.join(dirpath, "Restart_Passive_Scalar.bin")
    PS = rd("Restart_Passive_Scalar.bin").reshape(shape) if os.path.exists(ps) else None
    return State(RU=RU, Rho=rd("Restart_Rho.bin").reshape(shape),
                 P=rd("Restart_P.bin").reshape(shape), part=part, P0=float(tok[0]),
                 T_cur=float(tok[1]), num_timestep=int(tok[2]), PS=PS)


def passive_scalar(p: Params, seed: int) -> np.ndarray:
    """A smooth random scalar field at the cell centres: a few low Fourier modes."""
    rng = np.random.Generator(np.random.PCG64(1000 + seed))
    z, y, x = np.meshgrid((np.arange(p.Nz) + 0.5) * (p.Lz / p.Nz),
                          (np.arange(p.Ny) + 0.5) * (p.Ly / p.Ny),
                          (np.arange(p.Nx) + 0.5) * (p.Lx / p.Nx), indexing="ij")
    f = np.zeros((p.Nz, p.Ny, p.Nx))
    for _ in range(6):
        k = rng.integers(-3, 4, size=3)
        ph = rng.uniform(0, 2 * np.pi)
        f += rng.standard_normal() * np.cos(k[0] * 2 * np.pi / p.Lx * x +
                                            k[1] * 2 * np.pi / p.Ly * y +
                                            k[2] * 2 * np.pi / p.Lz * z + ph)
    return f
