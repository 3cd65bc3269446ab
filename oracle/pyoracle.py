"""CPU ORACLE bindings - TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module, and only as the checker (or the timed CPU baseline).  It wraps
  * ``_build/liboracle.so`` - the C restatement of the reference substep
    (tpm_oracle.c), and
  * ``_ref/tpm_ref``        - the reference's own sources compiled here with
    the single-rank stand-ins in refshim/ (built only where the reference
    sources exist).
"""
from __future__ import annotations

import ctypes
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(REPO, "triplyperiodic-modified_gb300"))

from tpm.params import Params, TpmScalars, TpmStats  # noqa: E402
from tpm import inputs  # noqa: E402

LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_BIN = os.path.join(HERE, "_ref", "tpm_ref")

F = dict(RU=0, RU_INT=1, RU_NEW=2, RU_NP1=3, RHO=4, RHO_INT=5, RHO_NEW=6, RHO_NP1=7, P=8,
         C=9, Q=10, FP=11, RHS_POIS=12, DIVERGENCE=13, PASSIVE_SCALAR=14)
VECTOR_FIELDS = {"RU", "RU_INT", "RU_NEW", "RU_NP1", "FP"}


def build(quiet: bool = True) -> None:
    """Compile liboracle.so (and the reference binary when its sources exist)."""
    out = subprocess.DEVNULL if quiet else None
    subprocess.check_call(["make", "-C", HERE, "-s"], stdout=out)
    has_ref = subprocess.call(["make", "-C", HERE, "-s", "has-ref"], stdout=subprocess.DEVNULL,
                              stderr=subprocess.DEVNULL) == 0
    if has_ref:
        subprocess.check_call(["make", "-C", HERE, "-s", "-j8", "ref"], stdout=out,
                              stderr=subprocess.DEVNULL if quiet else None)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        vp, dp, ip = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_int
        L.orc_create.restype = vp
        L.orc_create.argtypes = [vp, ctypes.c_int64]
        L.orc_destroy.argtypes = [vp]
        L.orc_set_field.argtypes = [vp, ip, dp]
        L.orc_get_field.argtypes = [vp, ip, dp]
        L.orc_set_particles.argtypes = [vp, ip] + [dp] * 7 + [ctypes.POINTER(ctypes.c_int32)]
        L.orc_get_particles.argtypes = [vp, ip] + [dp] * 7 + [ctypes.POINTER(ctypes.c_int32)]
        L.orc_get_particle_rhs_t.argtypes = [vp, dp]
        L.orc_set_particle_tau.argtypes = [vp, dp]
        L.orc_set_scalars.argtypes = [vp, ctypes.c_double, ctypes.c_double, ctypes.c_int64]
        L.orc_get_scalars.argtypes = [vp, vp]
        L.orc_initialize.argtypes = [vp]
        L.orc_substep.argtypes = [vp, ip, ip]
        L.orc_end_step.argtypes = [vp]
        L.orc_step.argtypes = [vp, ip]
        L.orc_poisson_solve.restype = ip
        L.orc_poisson_solve.argtypes = [vp, dp, dp, dp, ip, ctypes.c_double, dp]
        L.orc_statistics.argtypes = [vp, vp]
        L.orc_rdf_pairs.argtypes = [dp, dp, dp, ctypes.c_int64, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_double, ctypes.c_double, ip,
                                    ctypes.POINTER(ctypes.c_uint64)]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Oracle:
    """The C restatement driven like the reference grid (one box, one core)."""

    def __init__(self, p: Params, npart: int):
        self.p = p
        self.npart = npart
        self._cp = p.to_c()
        self.h = lib().orc_create(ctypes.byref(self._cp), npart)

    def close(self):
        if self.h:
            lib().orc_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    # ---- state ----
    def _shape(self, name):
        s = (self.p.Nz, self.p.Ny, self.p.Nx)
        return ((3,) + s) if name in VECTOR_FIELDS else s

    def set_field(self, name, a):
        a = np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
        lib().orc_set_field(self.h, F[name], _dp(a))

    def get_field(self, name):
        a = np.empty(self._shape(name))
        lib().orc_get_field(self.h, F[name], _dp(a))
        return a

    def set_particles(self, part, pset=0):
        arrs = [np.ascontiguousarray(part[q], dtype=np.float64) for q in inputs.PQ]
        flag = np.ascontiguousarray(part["flag"], dtype=np.int32)
        lib().orc_set_particles(self.h, pset, *[_dp(a) for a in arrs],
                                flag.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))

    def get_particles(self, pset=0):
        out = {q: np.empty(self.npart) for q in inputs.PQ}
        out["flag"] = np.empty(self.npart, dtype=np.int32)
        lib().orc_get_particles(self.h, pset, *[_dp(out[q]) for q in inputs.PQ],
                                out["flag"].ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
        return out

    def get_rhs_t(self):
        a = np.empty(self.npart)
        lib().orc_get_particle_rhs_t(self.h, _dp(a))
        return a

    def set_tau(self, tau):
        if tau is None:
            lib().orc_set_particle_tau(self.h, None)
        else:
            t = np.ascontiguousarray(tau, dtype=np.float64)
            lib().orc_set_particle_tau(self.h, _dp(t))

    def scalars(self):
        s = TpmScalars()
        lib().orc_get_scalars(self.h, ctypes.byref(s))
        return s.as_dict()

    def load(self, s: inputs.State):
        self.set_field("RU", s.RU)
        self.set_field("RHO", s.Rho)
        self.set_field("P", s.P)
        if s.PS is not None:
            self.set_field("PASSIVE_SCALAR", s.PS)
        self.set_particles(s.part, 0)
        lib().orc_set_scalars(self.h, s.P0, s.T_cur, s.num_timestep)
        if s.tau is not None:
            self.set_tau(s.tau)

    # ---- stepping ----
    def initialize(self):
        lib().orc_initialize(self.h)

    def substep(self, stage, with_particles=True):
        lib().orc_substep(self.h, stage, int(with_particles))

    def end_step(self):
        lib().orc_end_step(self.h)

    def step(self, with_particles=True):
        lib().orc_step(self.h, int(with_particles))

    def statistics(self):
        s = TpmStats()
        lib().orc_statistics(self.h, ctypes.byref(s))
        return s.as_dict()

    def poisson_solve(self, C3, P, RHS, max_it, eps):
        C3 = np.ascontiguousarray(C3, dtype=np.float64)
        P = np.ascontiguousarray(P, dtype=np.float64).copy()
        RHS = np.ascontiguousarray(RHS, dtype=np.float64)
        err = ctypes.c_double(0)
        it = lib().orc_poisson_solve(self.h, _dp(C3), _dp(P), _dp(RHS), max_it, eps,
                                     ctypes.byref(err))
        return P, it, err.value


def rdf_pairs(x, y, z, L, r_max, nbins):
    """All-pairs (O(Np^2), C) histogram of minimum-image distances."""
    x, y, z = (np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, z))
    out = np.zeros(nbins, dtype=np.uint64)
    lib().orc_rdf_pairs(_dp(x), _dp(y), _dp(z), x.shape[0], float(L[0]), float(L[1]),
                        float(L[2]), float(r_max), int(nbins),
                        out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)))
    return out


def face_velocity(RU, Rho):
    """u_d = RU_d / I_C2F_d(Rho), I_C2F(f)[i] = (f[i] + f[i-1]) * 0.5 (tensor0.cpp:268-362)."""
    U = np.empty_like(RU)
    for d, ax in enumerate((2, 1, 0)):  # x, y, z are the last, middle, first array axes
        U[d] = RU[d] / ((Rho + np.roll(Rho, 1, axis=ax)) * 0.5)
    return U


def spectrum(p: Params, RU, Rho):
    """Shell-summed energy spectrum of the face velocity (tpm_spectrum's definition):
    E[s] = sum over wave vectors with nint(|k|/dk) = s of |u_hat|^2/2, u_hat = DFT/N^3."""
    U = face_velocity(RU, Rho)
    ntot = p.Nx * p.Ny * p.Nz
    e = np.zeros((p.Nz, p.Ny, p.Nx // 2 + 1))
    for d in range(3):
        F = np.fft.rfftn(U[d]) / ntot
        e += F.real * F.real + F.imag * F.imag
    w = np.full(p.Nx // 2 + 1, 1.0)
    w[0] = 0.5
    w[-1] = 0.5
    e *= w[None, None, :]
    two_pi = 2 * 3.141592653589793
    kx0, ky0, kz0 = two_pi / p.Lx, two_pi / p.Ly, two_pi / p.Lz
    dk = min(kx0, ky0, kz0)
    kx = np.arange(p.Nx // 2 + 1) * kx0
    ky = np.where(np.arange(p.Ny) <= p.Ny // 2, np.arange(p.Ny), np.arange(p.Ny) - p.Ny) * ky0
    kz = np.where(np.arange(p.Nz) <= p.Nz // 2, np.arange(p.Nz), np.arange(p.Nz) - p.Nz) * kz0
    km = np.sqrt(kx[None, None, :] ** 2 + ky[None, :, None] ** 2 + kz[:, None, None] ** 2)
    shell = np.floor(km / dk + 0.5).astype(np.int64)
    return np.bincount(shell.ravel(), weights=e.ravel()), dk


# ---------------------------------------------------------------- reference
def have_reference() -> bool:
    return os.path.exists(REF_BIN)


# grid::Statistics output files (grid.cpp:32-57) -> tpm_stats members
STAT_FILES = {"Tg": "Tg_mean", "Tp": "Tp_mean", "HT": "HT_mean", "RU": "TKE2",
              "TKE_U": "TKE_U", "TKE_V": "TKE_V", "TKE_W": "TKE_W", "P0": "P0",
              "C_Max": "C_max", "C_Min": "C_min", "C_Mean": "C_mean", "Rho_Max": "Rho_max",
              "Rho_Min": "Rho_min", "Rho_Mean": "Rho_mean", "Max_CFL_U": "Gas_CFL_Max"}


def run_reference(p: Params, s: inputs.State, nsteps: int, substeps: int = 0,
                  as_shipped: bool = False, workdir: str | None = None,
                  stats: bool = False) -> dict:
    """Run the reference build on state `s`; returns its dumped state (and,
    with stats, the per-step grid::Statistics values it wrote)."""
    tmp = workdir or tempfile.mkdtemp(prefix="tpm_ref_")
    inputs.write_restart(tmp, p, s, statistics=stats)
    out = os.path.join(tmp, "out")
    os.makedirs(out, exist_ok=True)
    cmd = [REF_BIN, "deck.txt", str(nsteps), out]
    if as_shipped:
        cmd.append("--as-shipped")
    if substeps:
        cmd += ["--substeps", str(substeps)]
    if stats:
        cmd.append("--stats")
    res = subprocess.run(cmd, cwd=tmp, capture_output=True, text=True, check=True)
    info = json.loads(res.stdout.strip().splitlines()[-1])
    d = read_reference_dump(p, out, info)
    if stats:
        d["stats"] = {}
        for fname, key in STAT_FILES.items():
            rows = np.loadtxt(os.path.join(tmp, fname + ".dat"), ndmin=2)
            d["stats"][key] = rows[:, 1]
            d["stats"]["T_cur"] = rows[:, 0]
    return d


def read_reference_dump(p: Params, out: str, info: dict | None = None) -> dict:
    shape = (p.Nz, p.Ny, p.Nx)
    rd = lambda n, dt=np.float64: np.fromfile(os.path.join(out, n), dtype=dt)
    d = {"info": info}
    for name in ("RU", "RU_int", "RU_np1", "RU_new", "RHS_RU"):
        d[name] = rd(name + ".bin").reshape((3,) + shape)
    for name in ("Rho", "Rho_new", "Rho_np1", "P", "C", "RHS_Part_Temp", "RHS_Pois",
                 "divergence"):
        d[name] = rd(name + ".bin").reshape(shape)
    if os.path.exists(os.path.join(out, "Passive_Scalar.bin")):
        d["Passive_Scalar"] = rd("Passive_Scalar.bin").reshape(shape)
    part = {q: rd(f"Part_{q}.bin") for q in inputs.PQ}
    part["flag"] = rd("Part_flag.bin", np.int32)
    part["RHS_T"] = rd("Part_RHS_T.bin")
    for q in inputs.PQ:
        part[q + "_np1"] = rd(f"Part_{q}_np1.bin")
        part[q + "_int"] = rd(f"Part_{q}_int.bin")
    # restore id order (the reference's migration reorders particles)
    order = np.argsort(part["flag"], kind="stable")
    d["part"] = {k: v[order] for k, v in part.items()}
    with open(os.path.join(out, "scalars.txt")) as f:
        tok = f.read().split()
    d["P0"], d["P0_np1"], d["P0_int"], d["T_cur"] = map(float, tok[:4])
    d["num_timestep"], d["np"], d["steps"] = int(tok[4]), int(tok[5]), int(tok[6])
    d["seconds"] = float(tok[7])
    return d
