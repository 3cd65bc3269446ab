"""ctypes binding of libtpm.so (include/tpm.h) and a ``Grid`` facade that
mirrors the reference grid's public surface (grid.h:109-136): the same
method names run the same steps on the GPU.

There is no CPU fallback: constructing a context without the built library
or without a CUDA device raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import inputs
from .params import Params, TpmParams, TpmScalars, TpmStats

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG, "lib", "libtpm.so")

FIELD = dict(RU=0, RU_INT=1, RU_NEW=2, RU_NP1=3, RHO=4, RHO_INT=5, RHO_NEW=6, RHO_NP1=7, P=8,
             C=9, Q=10, FP=11, RHS_POIS=12, DIVERGENCE=13, PASSIVE_SCALAR=14)
VECTOR = {"RU", "RU_INT", "RU_NEW", "RU_NP1", "FP"}
PSET = dict(base=0, int=1, new=2, np1=3)
OPT_STORE_DIVERGENCE = 1
OPT_DIV_RESIDUAL_EVERY_STAGE = 2
OPT_CUDA_GRAPH = 3
OPT_FFT_TMA = 4
OPT_FUSED_DEPOSITS = 5
STATUS = {0: "TPM_OK", -1: "TPM_ERR_ARG", -2: "TPM_ERR_CUDA", -3: "TPM_ERR_TIMEOUT",
          -4: "TPM_ERR_NONFINITE", -5: "TPM_ERR_UNSUPPORTED", -6: "TPM_ERR_STATE",
          -7: "TPM_ERR_NOMEM"}

# every entry point include/tpm.h declares: name -> (restype, argtypes)
_vp, _dp, _ip = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int32)
_i, _d, _i64 = ctypes.c_int, ctypes.c_double, ctypes.c_int64
SIGNATURES = {
    "tpm_abi_version": (_i, []),
    "tpm_create": (_i, [_vp, _i64, ctypes.POINTER(_vp)]),
    "tpm_destroy": (_i, [_vp]),
    "tpm_last_error": (ctypes.c_char_p, [_vp]),
    "tpm_upload_field": (_i, [_vp, _i, _dp]),
    "tpm_download_field": (_i, [_vp, _i, _dp]),
    "tpm_upload_particles": (_i, [_vp, _i] + [_dp] * 7 + [_ip]),
    "tpm_download_particles": (_i, [_vp, _i] + [_dp] * 7 + [_ip]),
    "tpm_download_particle_rhs_t": (_i, [_vp, _dp]),
    "tpm_upload_particle_rhs_t": (_i, [_vp, _dp]),
    "tpm_set_particle_tau": (_i, [_vp, _dp]),
    "tpm_resume": (_i, [_vp]),
    "tpm_load_state": (_i, [_vp, _dp, _dp, _dp, _dp, ctypes.POINTER(_dp), _dp, _d, _d, _i64]),
    "tpm_save_state": (_i, [_vp, _dp, _dp, _dp, _dp, ctypes.POINTER(_dp), _dp, _vp]),
    "tpm_step_state": (_i, [_vp, _dp, _dp, _dp, _dp, ctypes.POINTER(_dp), _dp, ctypes.c_double,
                            ctypes.c_double, ctypes.c_int64, _dp, _dp, _dp, _dp,
                            ctypes.POINTER(_dp), _dp, _vp]),
    "tpm_statistics": (_i, [_vp, _vp]),
    "tpm_spectrum_shells": (_i, [_vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)]),
    "tpm_spectrum": (_i, [_vp, ctypes.POINTER(ctypes.c_double), _i]),
    "tpm_rdf": (_i, [_vp, ctypes.c_double, _i, ctypes.POINTER(ctypes.c_uint64),
                     ctypes.POINTER(ctypes.c_double)]),
    "tpm_write_restart": (_i, [_vp, ctypes.c_char_p]),
    "tpm_read_restart": (_i, [_vp, ctypes.c_char_p]),
    "tpm_store": (_i, [_vp, ctypes.c_char_p]),
    "tpm_stream": (_vp, [_vp]),
    "tpm_set_scalars": (_i, [_vp, _d, _d, _i64]),
    "tpm_get_scalars": (_i, [_vp, _vp]),
    "tpm_initialize": (_i, [_vp]),
    "tpm_substep": (_i, [_vp, _i]),
    "tpm_end_step": (_i, [_vp]),
    "tpm_param_update": (_i, [_vp]),
    "tpm_update_rho": (_i, [_vp, _i]),
    "tpm_update_p0": (_i, [_vp, _i]),
    "tpm_update_particle": (_i, [_vp, _i]),
    "tpm_update_passive_scalar": (_i, [_vp, _i]),
    "tpm_update_ru_wop": (_i, [_vp, _i]),
    "tpm_compute_div_u_new": (_i, [_vp, _i]),
    "tpm_compute_rhs_pois": (_i, [_vp, _i]),
    "tpm_solve_poisson": (_i, [_vp, _i]),
    "tpm_update_ru_wp": (_i, [_vp, _i]),
    "tpm_time_advance_rk4": (_i, [_vp, _i]),
    "tpm_make_mean_u0": (_i, [_vp]),
    "tpm_time_advance": (_i, [_vp]),
    "tpm_step": (_i, [_vp]),
    "tpm_run": (_i, [_vp, _i]),
    "tpm_sync": (_i, [_vp]),
    "tpm_poisson_solve": (_i, [_vp, _dp, _dp, _dp, _i, _d, ctypes.POINTER(_i), _dp]),
    "tpm_set_option": (_i, [_vp, _i, _i]),
    "tpm_poisson_solve_noalloc": (_i, [_i, _i, _i, _d, _d, _d, _vp, _vp, _vp, _i, _d, _vp,
                                       ctypes.POINTER(_i), _dp]),
    "tpm_measure_fp64_peak": (_i, [_dp]),
    "tpm_profile_enable": (_i, [_vp, _i]),
    "tpm_profile_report": (_i, [_vp, ctypes.c_char_p, _i, ctypes.POINTER(_i), _dp, _i]),
    "tpm_profile_reset": (_i, [_vp]),
    "tpm_launch_count": (_i64, [_vp]),
    "tpm_autotune": (_i, [_vp, ctypes.POINTER(_i)]),
    "tpm_set_fft_tiles": (_i, [_vp, ctypes.POINTER(_i)]),
    "tpm_adjoint_run": (_i, [_vp, _i, _i, _d, _d, _dp, _dp, _dp, _dp]),
    "tpm_batch_create": (_i, [_vp, ctypes.POINTER(_i64), _i, ctypes.POINTER(_vp)]),
    "tpm_batch_destroy": (_i, [_vp]),
    "tpm_batch_last_error": (ctypes.c_char_p, [_vp]),
    "tpm_batch_box": (_vp, [_vp, _i]),
    "tpm_batch_autotune": (_i, [_vp]),
    "tpm_batch_run": (_i, [_vp, _i, _i]),
    "tpm_batch_sync": (_i, [_vp]),
}

_lib = None


def load_library(path: str = LIB_PATH):
    """dlopen libtpm.so and declare every entry point (raises if absent)."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is not built: run __graft_entry__.build() first")
        L = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


class TpmError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


def _dptr(a):
    return a.ctypes.data_as(_dp)


class Context:
    """One periodic box resident on the current CUDA device."""

    def __init__(self, p: Params, npart: int):
        self.L = load_library()
        self.p = p
        self.npart = int(npart)
        self._cp = p.to_c()
        h = _vp()
        rc = self.L.tpm_create(ctypes.byref(self._cp), self.npart, ctypes.byref(h))
        self.h = h
        if rc != 0:
            msg = self.L.tpm_last_error(h).decode() if h.value else "create failed"
            self.L.tpm_destroy(h)
            self.h = None
            raise TpmError(rc, msg)

    @classmethod
    def borrowed(cls, handle, p: Params, npart: int, owner):
        """A view of a context owned elsewhere (a box of a Batch)."""
        self = cls.__new__(cls)
        self.L = load_library()
        self.p = p
        self.npart = int(npart)
        self._cp = p.to_c()
        self.h = _vp(handle)
        self._owner = owner
        return self

    def _check(self, rc):
        if rc != 0:
            raise TpmError(rc, self.L.tpm_last_error(self.h).decode())
        return rc

    def close(self):
        if getattr(self, "_owner", None) is not None:
            self.h = None
            return
        if getattr(self, "h", None):
            self.L.tpm_destroy(self.h)
            self.h = None

    def set_graph(self, on=True):
        self.set_option(OPT_CUDA_GRAPH, int(on))

    def adjoint(self, nsteps, checkpoint_every=20, w_tke=1.0, w_cvar=0.0, grad_ru0=True):
        """J and (dJ/dRU0, dJ/dA, dJ/dtau) by the discrete adjoint (tpm_adjoint_run)."""
        J, gA, gt = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        g = np.empty((3, self.p.Nz, self.p.Ny, self.p.Nx)) if grad_ru0 else None
        self._check(self.L.tpm_adjoint_run(self.h, int(nsteps), int(checkpoint_every),
                                           float(w_tke), float(w_cvar), ctypes.byref(J),
                                           _dptr(g) if g is not None else None,
                                           ctypes.byref(gA), ctypes.byref(gt)))
        return J.value, g, gA.value, gt.value

    def autotune(self):
        """FFT tiles: [pencils x, y, z, threads x, y, z]."""
        pens = (_i * 6)()
        self._check(self.L.tpm_autotune(self.h, pens))
        return list(pens)

    def set_fft_tiles(self, tiles):
        """Fix the FFT tiles ([pencils x, y, z, threads x, y, z], as autotune
        returns them) instead of searching."""
        arr = (_i * 6)(*[int(t) for t in tiles])
        self._check(self.L.tpm_set_fft_tiles(self.h, arr))

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- fields ----
    def _shape(self, name):
        s = (self.p.Nz, self.p.Ny, self.p.Nx)
        return ((3,) + s) if name in VECTOR else s

    def upload_field(self, name, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        if a.size != int(np.prod(self._shape(name))):
            raise ValueError(f"{name}: expected {self._shape(name)}, got {a.shape}")
        self._check(self.L.tpm_upload_field(self.h, FIELD[name], _dptr(a)))

    def download_field(self, name, out=None):
        a = np.empty(self._shape(name)) if out is None else out
        if a.dtype != np.float64 or not a.flags.c_contiguous or a.size != np.prod(self._shape(name)):
            raise ValueError(f"{name}: bad output buffer")
        self._check(self.L.tpm_download_field(self.h, FIELD[name], _dptr(a)))
        return a

    # ---- particles ----
    def upload_particles(self, part, pset="base"):
        arrs = [np.ascontiguousarray(part[q], dtype=np.float64) for q in inputs.PQ]
        flag = np.ascontiguousarray(part["flag"], dtype=np.int32)
        self._check(self.L.tpm_upload_particles(self.h, PSET[pset], *[_dptr(a) for a in arrs],
                                                flag.ctypes.data_as(_ip)))

    def download_particles(self, pset="base", out=None):
        if out is None:
            out = {q: np.empty(self.npart) for q in inputs.PQ}
            out["flag"] = np.empty(self.npart, dtype=np.int32)
        self._check(self.L.tpm_download_particles(self.h, PSET[pset],
                                                  *[_dptr(out[q]) for q in inputs.PQ],
                                                  out["flag"].ctypes.data_as(_ip)))
        return out

    def download_rhs_t(self, out=None):
        a = np.empty(self.npart) if out is None else out
        self._check(self.L.tpm_download_particle_rhs_t(self.h, _dptr(a)))
        return a

    def upload_rhs_t(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        self._check(self.L.tpm_upload_particle_rhs_t(self.h, _dptr(a)))

    # ---- diagnostics ----
    def statistics(self):
        s = TpmStats()
        self._check(self.L.tpm_statistics(self.h, ctypes.byref(s)))
        return s.as_dict()

    def spectrum(self):
        n, dk = ctypes.c_int(0), ctypes.c_double(0)
        self._check(self.L.tpm_spectrum_shells(self.h, ctypes.byref(n), ctypes.byref(dk)))
        E = np.zeros(n.value)
        self._check(self.L.tpm_spectrum(self.h, E.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                        n.value))
        return E, dk.value

    def rdf(self, r_max, nbins):
        pairs = np.zeros(nbins, dtype=np.uint64)
        g = np.zeros(nbins)
        self._check(self.L.tpm_rdf(self.h, float(r_max), int(nbins),
                                   pairs.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                                   g.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return pairs, g

    def write_restart(self, dirpath):
        self._check(self.L.tpm_write_restart(self.h, dirpath.encode()))

    def read_restart(self, dirpath):
        self._check(self.L.tpm_read_restart(self.h, dirpath.encode()))

    def store(self, dirpath):
        self._check(self.L.tpm_store(self.h, dirpath.encode()))

    def resume(self):
        self._check(self.L.tpm_resume(self.h))

    def stream(self):
        return self.L.tpm_stream(self.h)

    # ---- exact step-boundary state (what tpm_resume needs) ----
    STATE_FIELDS = ("RU", "RU_INT", "RHO", "P")

    def download_state(self, out=None):
        """Step-boundary state (tpm_save_state); with `out` (a previous result,
        e.g. in pinned host memory) the arrays are filled in place."""
        o = out or {}
        st = {}
        for f in self.STATE_FIELDS:
            a = o.get(f)
            st[f] = a if a is not None else np.empty(self._shape(f))
        part = o.get("part") or {q: np.empty(self.npart) for q in inputs.PQ}
        rhs_t = o.get("RHS_T")
        rhs_t = rhs_t if rhs_t is not None else np.empty(max(self.npart, 1))
        ptrs = (_dp * 7)(*[_dptr(part[q]) for q in inputs.PQ]) if self.npart else None
        sc = TpmScalars()
        self._check(self.L.tpm_save_state(self.h, *[_dptr(st[f]) for f in self.STATE_FIELDS],
                                          ptrs, _dptr(rhs_t), ctypes.byref(sc)))
        st["part"] = part if self.npart else None
        st["RHS_T"] = rhs_t if self.npart else None
        st["scalars"] = sc.as_dict()
        return st

    def upload_state(self, st):
        """Loads a state from download_state and resumes (tpm_load_state)."""
        arrs = [np.ascontiguousarray(st[f], dtype=np.float64) for f in self.STATE_FIELDS]
        if self.npart:
            part = [np.ascontiguousarray(st["part"][q], dtype=np.float64) for q in inputs.PQ]
            ptrs = (_dp * 7)(*[_dptr(a) for a in part])
            rhs_t = np.ascontiguousarray(st["RHS_T"], dtype=np.float64)
        else:
            ptrs, rhs_t = None, np.zeros(1)
        sc = st["scalars"]
        self._check(self.L.tpm_load_state(self.h, *[_dptr(a) for a in arrs], ptrs, _dptr(rhs_t),
                                          float(sc["P0"]), float(sc["T_cur"]),
                                          int(sc["num_timestep"])))

    def step_state(self, st, out=None):
        """One step of a host-resident state (tpm_step_state: load, step and
        save in one call, the transfers overlapping the step); `out` (e.g. `st`
        itself) receives the new state, in place when given."""
        out = out if out is not None else {
            **{f: np.empty(self._shape(f)) for f in self.STATE_FIELDS},
            "part": {q: np.empty(self.npart) for q in inputs.PQ} if self.npart else None,
            "RHS_T": np.empty(max(self.npart, 1)) if self.npart else None}
        for f in self.STATE_FIELDS:
            for d in (st, out):
                a = d[f]
                if not (a.flags["C_CONTIGUOUS"] and a.dtype == np.float64):
                    raise ValueError(f"{f}: contiguous float64 arrays only")
        if self.npart:
            pin = (_dp * 7)(*[_dptr(st["part"][q]) for q in inputs.PQ])
            pout = (_dp * 7)(*[_dptr(out["part"][q]) for q in inputs.PQ])
            rin, rout = _dptr(st["RHS_T"]), _dptr(out["RHS_T"])
        else:
            pin = pout = None
            rin = rout = _dptr(np.zeros(1))
        sc_in = st["scalars"]
        sc = TpmScalars()
        self._check(self.L.tpm_step_state(
            self.h, *[_dptr(st[f]) for f in self.STATE_FIELDS], pin, rin, float(sc_in["P0"]),
            float(sc_in["T_cur"]), int(sc_in["num_timestep"]),
            *[_dptr(out[f]) for f in self.STATE_FIELDS], pout, rout, ctypes.byref(sc)))
        out["scalars"] = sc.as_dict()
        return out

    def set_tau(self, tau):
        if tau is None:
            self._check(self.L.tpm_set_particle_tau(self.h, None))
        else:
            t = np.ascontiguousarray(tau, dtype=np.float64)
            self._check(self.L.tpm_set_particle_tau(self.h, _dptr(t)))

    # ---- scalars / control ----
    def set_scalars(self, P0, T_cur=0.0, num_timestep=0):
        self._check(self.L.tpm_set_scalars(self.h, P0, T_cur, num_timestep))

    def scalars(self):
        s = TpmScalars()
        self._check(self.L.tpm_get_scalars(self.h, ctypes.byref(s)))
        return s.as_dict()

    def set_option(self, opt, value):
        self._check(self.L.tpm_set_option(self.h, opt, int(value)))

    def load(self, s: inputs.State):
        self.upload_field("RU", s.RU)
        self.upload_field("RHO", s.Rho)
        self.upload_field("P", s.P)
        if s.PS is not None:
            self.upload_field("PASSIVE_SCALAR", s.PS)
        if self.npart:
            self.upload_particles(s.part, "base")
        self.set_scalars(s.P0, s.T_cur, s.num_timestep)
        if s.tau is not None:
            self.set_tau(s.tau)

    def initialize(self):
        self._check(self.L.tpm_initialize(self.h))

    def substep(self, stage):
        self._check(self.L.tpm_substep(self.h, stage))

    def end_step(self):
        self._check(self.L.tpm_end_step(self.h))

    def step(self):
        self._check(self.L.tpm_step(self.h))

    def run(self, nsteps):
        self._check(self.L.tpm_run(self.h, nsteps))

    def sync(self):
        self._check(self.L.tpm_sync(self.h))

    def poisson_solve(self, C3, P, RHS, max_it, eps):
        C3 = np.ascontiguousarray(C3, dtype=np.float64)
        P = np.ascontiguousarray(P, dtype=np.float64).copy()
        RHS = np.ascontiguousarray(RHS, dtype=np.float64)
        it = ctypes.c_int(0)
        err = ctypes.c_double(0)
        self._check(self.L.tpm_poisson_solve(self.h, _dptr(C3), _dptr(P), _dptr(RHS), max_it,
                                             eps, ctypes.byref(it), ctypes.byref(err)))
        return P, it.value, err.value

    # ---- profiling ----
    def profile(self, on=True):
        self._check(self.L.tpm_profile_enable(self.h, int(on)))

    def profile_reset(self):
        self._check(self.L.tpm_profile_reset(self.h))

    def profile_report(self):
        maxk, cap = 128, 8192
        names = ctypes.create_string_buffer(cap)
        launches = (ctypes.c_int * maxk)()
        ms = (ctypes.c_double * maxk)()
        k = self.L.tpm_profile_report(self.h, names, cap, launches, ms, maxk)
        if k < 0:
            self._check(k)
        out, off = {}, 0
        raw = names.raw
        for i in range(k):
            end = raw.index(b"\0", off)
            out[raw[off:end].decode()] = (int(launches[i]), float(ms[i]))
            off = end + 1
        return out

    def launch_count(self):
        return int(self.L.tpm_launch_count(self.h))


class Grid:
    """The reference grid's time-stepping surface (grid.h:112-136) on the GPU.

    The methods of the reference's loop (simulation.cpp:58-91) one by one -
    ``param_update``, ``Update_Rho``, ``Update_P0``, ``Update_Particle``,
    ``Update_Passive_Scalar``, ``Update_RU_WOP``, ``Compute_Div_U_new``,
    ``Compute_RHS_Pois``, ``Solve_Poisson``, ``Update_RU_WP``,
    ``TimeAdvance_RK4`` for stage ``RK4_count``, then ``RU_np1_make_mean_U0``
    and ``TimeAdvance`` - or whole pieces of it:
    ``Initialize``        -> grid::Initialize tail (grid.cpp:461-484)
    ``substep(k)``        -> Update_Rho ... TimeAdvance_RK4 for RK4_count = k
    ``end_step``          -> RU_np1.make_mean_U0 + grid::TimeAdvance
    ``step``              -> PARAM.update + 4 substeps + end of step
    """

    def __init__(self, p: Params, state: inputs.State):
        self.ctx = Context(p, state.npart)
        self.ctx.load(state)
        self.RK4_count = 0

    def Initialize(self):
        self.ctx.initialize()

    def _m(self, fn, *args):
        self.ctx._check(fn(self.ctx.h, *args))

    def param_update(self):
        self._m(self.ctx.L.tpm_param_update)

    def Update_Rho(self):
        self._m(self.ctx.L.tpm_update_rho, self.RK4_count)

    def Update_P0(self):
        self._m(self.ctx.L.tpm_update_p0, self.RK4_count)

    def Update_Particle(self):
        self._m(self.ctx.L.tpm_update_particle, self.RK4_count)

    def Update_Passive_Scalar(self):
        self._m(self.ctx.L.tpm_update_passive_scalar, self.RK4_count)

    def Update_RU_WOP(self):
        self._m(self.ctx.L.tpm_update_ru_wop, self.RK4_count)

    def Compute_Div_U_new(self):
        self._m(self.ctx.L.tpm_compute_div_u_new, self.RK4_count)

    def Compute_RHS_Pois(self):
        self._m(self.ctx.L.tpm_compute_rhs_pois, self.RK4_count)

    def Solve_Poisson(self):
        self._m(self.ctx.L.tpm_solve_poisson, self.RK4_count)

    def Update_RU_WP(self):
        self._m(self.ctx.L.tpm_update_ru_wp, self.RK4_count)

    def TimeAdvance_RK4(self):
        self._m(self.ctx.L.tpm_time_advance_rk4, self.RK4_count)

    def RU_np1_make_mean_U0(self):
        self._m(self.ctx.L.tpm_make_mean_u0)

    def TimeAdvance(self):
        self._m(self.ctx.L.tpm_time_advance)

    def substep(self, rk4_count):
        self.ctx.substep(rk4_count)

    def end_step(self):
        self.ctx.end_step()

    def step(self):
        self.ctx.step()

    @property
    def T_cur(self):
        return self.ctx.scalars()["T_cur"]

    @property
    def P0(self):
        return self.ctx.scalars()["P0"]

    def __getattr__(self, name):
        # field access by reference names: RU, RU_int, Rho, P, C, RHS_Part_Temp ...
        alias = {"RU": "RU", "RU_int": "RU_INT", "RU_new": "RU_NEW", "RU_np1": "RU_NP1",
                 "Rho": "RHO", "Rho_int": "RHO_INT", "Rho_new": "RHO_NEW", "Rho_np1": "RHO_NP1",
                 "P": "P", "C": "C", "RHS_Part_Temp": "Q", "RHS_Pois": "RHS_POIS",
                 "divergence": "DIVERGENCE"}
        if name in alias:
            return self.ctx.download_field(alias[name])
        raise AttributeError(name)


class Batch:
    """Independent boxes stepped together (tpm_batch_*)."""

    def __init__(self, params: list, nparts: list):
        self.L = load_library()
        self.params = list(params)
        self.nparts = [int(n) for n in nparts]
        arr = (TpmParams * len(params))(*[p.to_c() for p in params])
        nps = (_i64 * len(params))(*self.nparts)
        h = _vp()
        rc = self.L.tpm_batch_create(arr, nps, len(params), ctypes.byref(h))
        if rc != 0:
            raise TpmError(rc, "batch create failed")
        self.h = h
        self.boxes = [Context.borrowed(self.L.tpm_batch_box(h, i), p, n, self)
                      for i, (p, n) in enumerate(zip(self.params, self.nparts))]

    def _check(self, rc):
        if rc != 0:
            raise TpmError(rc, self.L.tpm_batch_last_error(self.h).decode())
        return rc

    def autotune(self):
        self._check(self.L.tpm_batch_autotune(self.h))

    def run(self, nsteps, graph=True):
        self._check(self.L.tpm_batch_run(self.h, int(nsteps), int(graph)))

    def sync(self):
        self._check(self.L.tpm_batch_sync(self.h))

    def close(self):
        if getattr(self, "h", None):
            for b in self.boxes:
                b.h = None
            self.L.tpm_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()
