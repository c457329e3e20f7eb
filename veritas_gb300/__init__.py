"""GB300-native Vlasov–Maxwell step (Veritas per-step path) — Python mirror of the C ABI.

The classes follow the reference's driver interface: :class:`SolverManager` stands in for
Veritas's ``SolverManager`` (SolverManager.hpp:5-19) with ``CalculateDt``, ``Advance``
and the state exchange used for checkpoints and parity tests.  Every call goes through
``libvx_cuda.so`` (declared in ``include/vx.h``); there is no CPU fallback — if the
library cannot be loaded, the first call into it raises.
"""
from __future__ import annotations

import ctypes
import os
import weakref
from dataclasses import dataclass, fields
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "libvx_cuda.so"

VX_ERRORS = {
    -1: "invalid argument",
    -2: "CUDA error",
    -3: "invalid state",
    -4: "I/O error",
    -5: "out of device memory",
    -6: "device wait timed out",
    -7: "unsupported",
}


class VxError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{VX_ERRORS.get(code, code)}: {msg}")
        self.code = code


class _Problem(ctypes.Structure):
    _fields_ = [
        ("lambda_", ctypes.c_double), ("L", ctypes.c_double),
        ("nx", ctypes.c_uint32), ("np", ctypes.c_uint32), ("Lfinest", ctypes.c_uint32), ("r", ctypes.c_uint32),
        ("pmax", ctypes.c_double), ("dens", ctypes.c_double),
        ("x1", ctypes.c_double), ("x2", ctypes.c_double), ("x3", ctypes.c_double), ("x4", ctypes.c_double),
        ("Te", ctypes.c_double), ("p0", ctypes.c_double), ("pert_amp", ctypes.c_double), ("pert_k", ctypes.c_double),
        ("a0", ctypes.c_double), ("fwhm", ctypes.c_double), ("delay", ctypes.c_double),
        ("cfl", ctypes.c_double), ("minEff", ctypes.c_double), ("crit", ctypes.c_double), ("sizeWeight", ctypes.c_double),
        ("quadDepth", ctypes.c_int32), ("precision", ctypes.c_int32),
        ("bdens", ctypes.c_double), ("bp0", ctypes.c_double), ("bTe", ctypes.c_double),
        ("poisson", ctypes.c_int32),
        ("mi", ctypes.c_double), ("iTe", ctypes.c_double), ("ipmax", ctypes.c_double),
        ("fast", ctypes.c_int32),
    ]


class _RequestResult(ctypes.Structure):
    _fields_ = [
        ("finished", ctypes.c_int32), ("steps_done", ctypes.c_int64), ("arrival", ctypes.c_double),
        ("admitted", ctypes.c_double), ("finish", ctypes.c_double), ("sim_time", ctypes.c_double),
        ("cells", ctypes.c_int64), ("device_bytes", ctypes.c_uint64), ("status", ctypes.c_int32),
        ("regrids", ctypes.c_int32), ("bound", ctypes.c_double), ("error", ctypes.c_char * 192),
    ]


# request states of the serving loop (VX_REQ_*)
REQ_WAITING, REQ_BUILDING, REQ_LIVE, REQ_DONE, REQ_CANCELLED, REQ_FAILED = range(6)


MAX_SPECIES = 8
MAX_MISC = 8
_D = ctypes.c_double
_I = ctypes.c_int32
_U = ctypes.c_uint32


class VxInput(ctypes.Structure):
    """vx_input (the reference's Input, Settings.hpp:4-11)."""
    _fields_ = [("minEfficiency", _D), ("dx", _D), ("k", _D), ("refinementCriteria", _D), ("cfl", _D),
                ("sizeWeight", _D), ("preLength", _D), ("postLength", _D), ("nx", _U), ("r", _U), ("Lfinest", _U),
                ("plasma_xl_bound", _D), ("plasma_xr_bound", _D), ("ntempEM", _I), ("tempEM", _D * MAX_MISC)]


class VxParticles(ctypes.Structure):
    """vx_particles (the reference's Particles, Settings.hpp:13-20)."""
    _fields_ = [("nspecies", _I), ("mass", _D * MAX_SPECIES), ("charge", _D * MAX_SPECIES), ("np", _U * MAX_SPECIES),
                ("dp", _D * MAX_SPECIES), ("pmin", _D * MAX_SPECIES), ("nmisc", _I * MAX_SPECIES),
                ("misc", (_D * MAX_MISC) * MAX_SPECIES)]


class VxOutput(ctypes.Structure):
    """vx_output (the reference's Output, Settings.hpp:22-33)."""
    _fields_ = [(n, _I) for n in ("time", "rectangleData", "charge", "energy", "potential", "EFieldLongitudinal",
                                  "EFieldTransverse", "BFieldTransverse", "AFieldSquared", "precision")]


class VxSettings(ctypes.Structure):
    """vx_settings (the reference's Settings, Settings.hpp:35-65)."""
    _fields_ = [(n, _D) for n in ("dx", "time", "minEfficiency", "preLength", "postLength", "refinementCriteria",
                                  "cfl", "sizeWeight", "plasma_xl_bound", "plasma_xr_bound")] + [
        ("nspecies", _I), ("m", _D * MAX_SPECIES), ("q", _D * MAX_SPECIES), ("m_inv", _D * MAX_SPECIES),
        ("dp", _D * MAX_SPECIES), ("fMax", _D * MAX_SPECIES), ("pmin", _D * MAX_SPECIES),
        ("ntemp", _I * MAX_SPECIES), ("temp", (_D * MAX_MISC) * MAX_SPECIES), ("ntempEM", _I),
        ("tempEM", _D * MAX_MISC), ("x_size_finest", _U), ("x_size", _U), ("refinementRatio", _U),
        ("maxDepth", _I), ("quadratureDepth", _I), ("p_size", _U * MAX_SPECIES),
        ("p_size_finest", _U * MAX_SPECIES)]


class VxHooks(ctypes.Structure):
    """vx_hooks: the user problem's callbacks (function pointers as void*)."""
    _fields_ = [("user", ctypes.c_void_p), ("initial_conditions", ctypes.c_void_p),
                ("settings_override", ctypes.c_void_p), ("initial_distribution", ctypes.c_void_p),
                ("get_by", ctypes.c_void_p), ("get_bz", ctypes.c_void_p), ("refinement_override", ctypes.c_void_p)]


# sub-step selection of vx_run_vlasov_stage
SUB_FLUX, SUB_LIMIT, SUB_UPDATE, SUB_COPY, SUB_ALL = 0x1, 0x2, 0x4, 0x8, 0xF


def _load() -> ctypes.CDLL:
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing: run `python -c 'import __graft_entry__ as g; g.build()'` first")
    lib = ctypes.CDLL(str(LIB_PATH))
    P = ctypes.POINTER
    vp = ctypes.c_void_p
    sig = {
        "vx_problem_defaults": (None, [P(_Problem)]),
        "vx_last_error": (ctypes.c_char_p, []),
        "vx_ctx_create": (ctypes.c_int, [ctypes.c_int, P(vp)]),
        "vx_ctx_destroy": (ctypes.c_int, [vp]),
        "vx_ctx_sync": (ctypes.c_int, [vp]),
        "vx_ctx_set_launch_mode": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int]),
        "vx_ctx_set_persistent": (ctypes.c_int, [vp, ctypes.c_int]),
        "vx_ctx_set_persistent_limit": (ctypes.c_int, [vp, ctypes.c_uint64, ctypes.c_int]),
        "vx_ctx_set_pipelined": (ctypes.c_int, [vp, ctypes.c_int]),
        "vx_ctx_kernel_launches": (ctypes.c_int, [vp, P(ctypes.c_uint64)]),
        "vx_run_create": (ctypes.c_int, [vp, P(_Problem), P(vp)]),
        "vx_run_destroy": (ctypes.c_int, [vp]),
        "vx_run_calculate_dt": (ctypes.c_int, [vp, P(ctypes.c_double)]),
        "vx_run_advance": (ctypes.c_int, [vp, ctypes.c_double]),
        "vx_runs_advance": (ctypes.c_int, [P(vp), P(ctypes.c_double), ctypes.c_int]),
        "vx_runs_calculate_dt": (ctypes.c_int, [P(vp), P(ctypes.c_double), ctypes.c_int]),
        "vx_runs_autotune": (ctypes.c_int, [P(vp), ctypes.c_int, P(ctypes.c_int), P(ctypes.c_int)]),
        "vx_server_create": (ctypes.c_int, [vp, ctypes.c_uint64, ctypes.c_int, P(vp)]),
        "vx_server_destroy": (ctypes.c_int, [vp]),
        "vx_server_clock": (ctypes.c_int, [vp, P(ctypes.c_double)]),
        "vx_server_submit": (ctypes.c_int, [vp, P(_Problem), ctypes.c_int64, ctypes.c_double, ctypes.c_char_p,
                                             P(ctypes.c_int64)]),
        "vx_server_step": (ctypes.c_int, [vp, P(ctypes.c_int), P(ctypes.c_int)]),
        "vx_server_result": (ctypes.c_int, [vp, ctypes.c_int64, P(_RequestResult)]),
        "vx_server_cancel": (ctypes.c_int, [vp, ctypes.c_int64]),
        "vx_server_set_regrid": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_double]),
        "vx_run_advance_fields": (ctypes.c_int, [vp, ctypes.c_double]),
        "vx_run_regrid": (ctypes.c_int, [vp]),
        "vx_error_weights": (ctypes.c_int, [P(_Problem), ctypes.c_int, ctypes.c_int, P(ctypes.c_double),
                                             P(ctypes.c_double)]),
        "vx_update_hierarchy": (ctypes.c_int, [P(_Problem), ctypes.c_int, P(ctypes.c_int32), ctypes.c_int,
                                                P(ctypes.c_int32), P(ctypes.c_int32), P(ctypes.c_int32), ctypes.c_int,
                                                P(ctypes.c_int)]),
        "vx_run_layout": (ctypes.c_int, [vp, P(ctypes.c_int32), ctypes.c_int, P(ctypes.c_int)]),
        "vx_run_time": (ctypes.c_int, [vp, P(ctypes.c_double)]),
        "vx_run_cell_count": (ctypes.c_int, [vp, P(ctypes.c_int64)]),
        "vx_run_load_state": (ctypes.c_int, [vp, ctypes.c_char_p]),
        "vx_run_save_state": (ctypes.c_int, [vp, ctypes.c_char_p]),
        "vx_run_get_field": (ctypes.c_int, [vp, ctypes.c_int, P(ctypes.c_double), P(ctypes.c_int64)]),
        "vx_run_write_fields": (ctypes.c_int, [vp, ctypes.c_char_p, ctypes.c_uint32, ctypes.c_int, ctypes.c_double]),
        "vx_run_write_rectangles": (ctypes.c_int, [vp, ctypes.c_char_p, ctypes.c_double]),
        "vx_ctx_timer_begin": (ctypes.c_int, [vp]),
        "vx_ctx_timer_end": (ctypes.c_int, [vp, P(ctypes.c_double)]),
        "vx_run_profile_kernels": (ctypes.c_int, [vp, ctypes.c_int, P(ctypes.c_double), ctypes.c_int, P(ctypes.c_int)]),
        "vx_ctx_flush_l2": (ctypes.c_int, [vp]),
        "vx_ctx_measure_fp64_peak": (ctypes.c_int, [vp, P(ctypes.c_double)]),
        "vx_ctx_measure_fp64_latency": (ctypes.c_int, [vp, P(ctypes.c_double), P(ctypes.c_double)]),
        "vx_host_alloc": (ctypes.c_int, [ctypes.c_size_t, P(vp)]),
        "vx_host_free": (ctypes.c_int, [vp]),
        "vx_run_state_size": (ctypes.c_int, [vp, P(ctypes.c_int64)]),
        "vx_run_step_host": (ctypes.c_int, [vp, P(ctypes.c_double), P(ctypes.c_double), ctypes.c_double]),
        "vx_run_state_to_host": (ctypes.c_int, [vp, P(ctypes.c_double)]),
        "vx_input_defaults": (None, [P(VxInput), P(VxParticles), P(VxOutput)]),
        "vx_run_create_hooks": (ctypes.c_int, [vp, P(VxHooks), ctypes.c_int, ctypes.c_int, P(vp)]),
        "vx_run_settings": (ctypes.c_int, [vp, P(VxSettings)]),
        "vx_run_moments": (ctypes.c_int, [vp]),
        "vx_run_poisson": (ctypes.c_int, [vp]),
        "vx_run_vlasov_stage": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_double, ctypes.c_uint]),
        "vx_run_update_time": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_double]),
        "vx_run_maxwell_stage": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_double]),
        "vx_run_flag": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, P(ctypes.c_int32), ctypes.c_int,
                                        P(ctypes.c_int)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


_CDLL = None


def lib() -> ctypes.CDLL:
    """The library, loaded on first use (raises if it is missing: there is no fallback)."""
    global _CDLL
    if _CDLL is None:
        _CDLL = _load()
    return _CDLL


class _LazyLib:
    """Forwards to the library, loading it on the first call: importing the package maps
    nothing, so a process that only reads problem definitions (the CPU reference arm of
    the benchmark) never loads the CUDA library."""

    def __getattr__(self, name):
        return getattr(lib(), name)


_lib = _LazyLib()


def _check(rc: int) -> None:
    if rc != 0:
        raise VxError(rc, (_lib.vx_last_error() or b"").decode())


@dataclass
class Problem:
    """Synthetic laser / plasma-slab problem (the hooks of the reference's veritas.cpp)."""

    lambda_: float = 1e-6
    L: float = 100.0
    nx: int = 2048
    np: int = 256
    Lfinest: int = 1
    r: int = 2
    pmax: float = 2.0
    dens: float = 0.01
    x1: float = 15.0
    x2: float = 20.0
    x3: float = 80.0
    x4: float = 85.0
    Te: float = 1.0
    p0: float = 0.0
    pert_amp: float = 0.0
    pert_k: float = 1.0
    a0: float = 1.0
    fwhm: float = 10.0
    delay: float = 10.0
    cfl: float = 0.5
    minEff: float = 0.75
    crit: float = 1e-6
    sizeWeight: float = 1.0
    quadDepth: int = 2
    precision: int = 64
    bdens: float = 0.0
    bp0: float = 0.0
    bTe: float = 1.0
    poisson: int = 0  # precision-64 runs: 0 the reference's LU rounding order, 1 the O(n) scan solve
    mi: float = 0.0     # mobile ions (second species) when > 0: mass / m_e
    iTe: float = 1.0    # ion temperature [keV]
    ipmax: float = 0.1  # ion momenta in [-ipmax, ipmax] m_i c
    fast: int = 0       # precision-64 runs: 1 = contracted FCT kernels (not the reference's rounding)

    def to_c(self) -> _Problem:
        p = _Problem()
        for f in fields(self):
            setattr(p, f.name, getattr(self, f.name))
        return p

    def harness_args(self) -> list[str]:
        """key=value arguments of the oracle harness for the same problem."""
        keys = ["L", "nx", "np", "r", "pmax", "dens", "x1", "x2", "x3", "x4", "Te", "p0", "pert_amp", "pert_k",
                "a0", "fwhm", "delay", "cfl", "minEff", "crit", "sizeWeight", "quadDepth", "bdens", "bp0", "bTe",
                "mi", "iTe", "ipmax"]
        out = [f"{k}={getattr(self, k)!r}" for k in keys]
        out.append(f"levels={self.Lfinest}")
        return out


class Context:
    """One GPU and one CUDA stream (vx_ctx)."""

    def __init__(self, device: int = 0):
        h = ctypes.c_void_p()
        _check(_lib.vx_ctx_create(device, ctypes.byref(h)))
        self._h = h
        self._runs = weakref.WeakSet()

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    def sync(self) -> None:
        _check(_lib.vx_ctx_sync(self._h))

    def set_launch_mode(self, graphs: bool = True, pdl: bool = True) -> None:
        """CUDA graph per step and programmatic dependent launch (both on by default)."""
        _check(_lib.vx_ctx_set_launch_mode(self._h, int(graphs), int(pdl)))

    def set_persistent(self, on: bool = True) -> None:
        """FP32 runs: three launches per RK stage (two persistent cooperative stage kernels
        around the Poisson solve) instead of one per sub-step; same bits."""
        _check(_lib.vx_ctx_set_persistent(self._h, int(on)))

    def set_persistent_limit(self, limit_ns: int = 2_000_000_000, phantom: int = 0) -> None:
        """Wait limit of the persistent kernels' grid barriers; phantom > 0 makes every wait
        run out (failure-path test)."""
        _check(_lib.vx_ctx_set_persistent_limit(self._h, int(limit_ns), int(phantom)))

    def set_pipelined(self, on: bool = True) -> None:
        """FP64 runs with the exact solve (alone or up to four together): moments, assembly
        and solve of each RK stage in one launch whose solve follows the moments as they
        finish (on by default); off runs the three kernels one after another.  Same bits."""
        _check(_lib.vx_ctx_set_pipelined(self._h, int(on)))

    def kernel_launches(self) -> int:
        v = ctypes.c_uint64()
        _check(_lib.vx_ctx_kernel_launches(self._h, ctypes.byref(v)))
        return int(v.value)

    def timer_begin(self) -> None:
        _check(_lib.vx_ctx_timer_begin(self._h))

    def timer_end(self) -> float:
        v = ctypes.c_double()
        _check(_lib.vx_ctx_timer_end(self._h, ctypes.byref(v)))
        return float(v.value)

    def flush_l2(self) -> None:
        _check(_lib.vx_ctx_flush_l2(self._h))

    def measure_fp64_latency(self) -> tuple[float, float]:
        """(cycles of a dependent multiply + subtract, extra cycles of a 64-bit shuffle)."""
        a, b = ctypes.c_double(), ctypes.c_double()
        _check(_lib.vx_ctx_measure_fp64_latency(self._h, ctypes.byref(a), ctypes.byref(b)))
        return float(a.value), float(b.value)

    def measure_fp64_peak(self) -> float:
        v = ctypes.c_double()
        _check(_lib.vx_ctx_measure_fp64_peak(self._h, ctypes.byref(v)))
        return float(v.value)

    def close(self) -> None:
        """Destroys the context after every solve still open on it."""
        if self._h:
            for r in list(self._runs):
                r.close()
            _check(_lib.vx_ctx_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# Output flags of the reference (Settings.hpp:22-33) -> VX_OUT_* bits of vx.h.
OUTPUT_BITS = {"charge": 0x01, "energy": 0x02, "potential": 0x04, "EFieldLongitudinal": 0x08,
               "EFieldTransverse": 0x10, "BFieldTransverse": 0x20, "AFieldSquared": 0x40, "time": 0x80}

FIELD_IDS = {"By": 0, "Bz": 1, "Ey": 2, "Ez": 3, "Ay": 4, "Az": 5, "a_squared": 6, "phi": 7, "charge": 8, "J": 9,
             "Ex": 10}


class SolverManager:
    """One independent solve on a context (the reference's SolverManager)."""

    def __init__(self, ctx: Context, problem: Problem | None, *, hooks: VxHooks | None = None, precision: int = 64,
                 poisson: int = 0):
        """`problem`: the built-in laser / plasma-slab problem; or problem=None and `hooks`
        (a user problem as C callbacks, vx_run_create_hooks) with its precision and
        Poisson solver.  The hooks struct and whatever its pointers reference must outlive
        the run."""
        self.ctx = ctx
        self.problem = problem
        h = ctypes.c_void_p()
        if problem is not None:
            _check(_lib.vx_run_create(ctx.handle, ctypes.byref(problem.to_c()), ctypes.byref(h)))
        else:
            if hooks is None:
                raise ValueError("give a problem or hooks")
            self._hooks = hooks
            _check(_lib.vx_run_create_hooks(ctx.handle, ctypes.byref(hooks), precision, poisson, ctypes.byref(h)))
        self._h = h
        ctx._runs.add(self)

    # ---- per-class calls (EMFieldSolver / Mesh / Settings steps of one RK stage)
    def moments(self) -> None:
        """EMFieldSolver::AssembleRhoAndJ."""
        _check(_lib.vx_run_moments(self._h))

    def poisson(self) -> None:
        """EMFieldSolver::UpdatePotential (phi, Ex0, E_x)."""
        _check(_lib.vx_run_poisson(self._h))

    def vlasov_stage(self, stage: int, dt: float, sub_mask: int = SUB_ALL) -> None:
        """Mesh::Advance(dt, stage) for every species (sub_mask: SUB_* bits)."""
        _check(_lib.vx_run_vlasov_stage(self._h, stage, float(dt), sub_mask))

    def update_time(self, stage: int, dt: float) -> None:
        """Settings::UpdateTime."""
        _check(_lib.vx_run_update_time(self._h, stage, float(dt)))

    def maxwell_stage(self, stage: int, dt: float) -> None:
        """EMFieldSolver::RGKStep."""
        _check(_lib.vx_run_maxwell_stage(self._h, stage, float(dt)))

    def flag(self, species: int, depth: int) -> list[tuple[int, int]]:
        """Mesh::getError of one level: the flagged (i, j) in the reference's order."""
        cnt = ctypes.c_int()
        _check(_lib.vx_run_flag(self._h, species, depth, None, 0, ctypes.byref(cnt)))
        buf = (ctypes.c_int32 * max(2, 2 * cnt.value))()
        _check(_lib.vx_run_flag(self._h, species, depth, buf, cnt.value, ctypes.byref(cnt)))
        return [(buf[2 * k], buf[2 * k + 1]) for k in range(cnt.value)]

    def settings(self) -> VxSettings:
        out = VxSettings()
        _check(_lib.vx_run_settings(self._h, ctypes.byref(out)))
        return out

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    def CalculateDt(self) -> float:
        v = ctypes.c_double()
        _check(_lib.vx_run_calculate_dt(self._h, ctypes.byref(v)))
        return float(v.value)

    def Advance(self, dt: float) -> None:
        _check(_lib.vx_run_advance(self._h, float(dt)))

    def AdvanceFields(self, dt: float) -> None:
        _check(_lib.vx_run_advance_fields(self._h, float(dt)))

    def reGrid(self) -> None:
        _check(_lib.vx_run_regrid(self._h))

    def layout(self) -> list[tuple[int, int, int, int, int, int]]:
        """(species, depth, x_pos, p_pos, n_x, n_p) of every patch, in level order."""
        cnt = ctypes.c_int()
        _check(_lib.vx_run_layout(self._h, None, 0, ctypes.byref(cnt)))
        buf = (ctypes.c_int32 * max(1, 6 * cnt.value))()
        _check(_lib.vx_run_layout(self._h, buf, cnt.value, ctypes.byref(cnt)))
        return [tuple(buf[6 * k:6 * k + 6]) for k in range(cnt.value)]

    @property
    def time(self) -> float:
        v = ctypes.c_double()
        _check(_lib.vx_run_time(self._h, ctypes.byref(v)))
        return float(v.value)

    def cell_count(self) -> int:
        v = ctypes.c_int64()
        _check(_lib.vx_run_cell_count(self._h, ctypes.byref(v)))
        return int(v.value)

    def load_state(self, path: str | os.PathLike) -> None:
        _check(_lib.vx_run_load_state(self._h, str(path).encode()))

    def save_state(self, path: str | os.PathLike) -> None:
        _check(_lib.vx_run_save_state(self._h, str(path).encode()))

    def fileOutput(self, t: float, directory: str | os.PathLike = "output", outputs=None, precision: int = 15) -> None:
        """SolverManager::fileOutput(t) (SolverManager.cpp:102-159): appends one record to
        each of the reference's text files under `directory` (created by the run's first
        call).  `outputs`: names from OUTPUT_BITS (default: all, as Output's defaults)."""
        mask = 0xFF if outputs is None else sum(OUTPUT_BITS[o] for o in set(outputs))
        _check(_lib.vx_run_write_fields(self._h, str(directory).encode(), mask, precision, t))

    def OutputRectangles(self, t: float, directory: str | os.PathLike = "output/rectangleData") -> None:
        """SolverManager::OutputRectangles(t) / Mesh::outputRectangleData (Mesh.cpp:877-902)."""
        _check(_lib.vx_run_write_rectangles(self._h, str(directory).encode(), t))

    def field(self, name: str) -> np.ndarray:
        n = ctypes.c_int64()
        fid = FIELD_IDS[name]
        _check(_lib.vx_run_get_field(self._h, fid, None, ctypes.byref(n)))
        out = np.empty(n.value, dtype=np.float64)
        _check(_lib.vx_run_get_field(self._h, fid, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.byref(n)))
        return out

    PROFILE_KERNELS = ["gamma", "faces", "flux", "ds_f2", "limR", "limC", "update", "moments", "assemble", "poisson",
                       "maxwell", "ghost", "iface", "csync", "moments_poisson"]

    def profile_kernels(self, reps: int = 5) -> dict:
        buf = (ctypes.c_double * 16)()
        cnt = ctypes.c_int()
        _check(_lib.vx_run_profile_kernels(self._h, reps, buf, 16, ctypes.byref(cnt)))
        return {self.PROFILE_KERNELS[i]: float(buf[i]) for i in range(cnt.value)}

    def state_size(self) -> int:
        v = ctypes.c_int64()
        _check(_lib.vx_run_state_size(self._h, ctypes.byref(v)))
        return int(v.value)

    def state_to_host(self, out: np.ndarray) -> None:
        _check(_lib.vx_run_state_to_host(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))

    def step_host(self, state_in: np.ndarray, state_out: np.ndarray, dt: float) -> None:
        dp = ctypes.POINTER(ctypes.c_double)
        _check(_lib.vx_run_step_host(self._h, state_in.ctypes.data_as(dp), state_out.ctypes.data_as(dp), float(dt)))

    def close(self) -> None:
        if self._h:
            _check(_lib.vx_run_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def error_weights(problem: Problem, species: int, depth: int) -> tuple[list[float], float]:
    """Rectangle error weights and refinement criterion (host only)."""
    w = (ctypes.c_double * 5)()
    crit = ctypes.c_double()
    _check(_lib.vx_error_weights(ctypes.byref(problem.to_c()), species, depth, w, ctypes.byref(crit)))
    return list(w), float(crit.value)


def update_hierarchy(problem: Problem, species: int, patches: list, flags: list) -> list[tuple]:
    """Mesh::updateHierarchy clustering on the host.

    patches: [(depth, x_pos, p_pos, n_x, n_p)] in level order; flags: per patch a list of
    flagged (i, j) in global level coordinates.  Returns the new patches as
    (depth, x_pos, p_pos, n_x, n_p, up, down, left, right)."""
    n = len(patches)
    pa = (ctypes.c_int32 * (5 * n))(*[v for p in patches for v in p])
    ptr = [0]
    for f in flags:
        ptr.append(ptr[-1] + len(f))
    fp = (ctypes.c_int32 * (n + 1))(*ptr)
    fij = (ctypes.c_int32 * max(1, 2 * ptr[-1]))(*[v for f in flags for c in f for v in c])
    cnt = ctypes.c_int()
    _check(_lib.vx_update_hierarchy(ctypes.byref(problem.to_c()), species, pa, n, fp, fij, None, 0, ctypes.byref(cnt)))
    out = (ctypes.c_int32 * max(1, 9 * cnt.value))()
    _check(_lib.vx_update_hierarchy(ctypes.byref(problem.to_c()), species, pa, n, fp, fij, out, cnt.value,
                                    ctypes.byref(cnt)))
    return [tuple(out[9 * k:9 * k + 9]) for k in range(cnt.value)]


class PinnedArray:
    """Page-locked float64 host buffer (cudaMallocHost through the C ABI)."""

    def __init__(self, n: int):
        p = ctypes.c_void_p()
        _check(_lib.vx_host_alloc(max(8, 8 * n), ctypes.byref(p)))
        self._p = p
        buf = (ctypes.c_double * n).from_address(p.value)
        self.array = np.frombuffer(buf, dtype=np.float64, count=n)

    def close(self) -> None:
        if self._p:
            self.array = None
            _check(_lib.vx_host_free(self._p))
            self._p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def advance_many(runs: list[SolverManager], dts: list[float]) -> None:
    """Advance several runs of one context together (batched launch per sub-step)."""
    arr = (ctypes.c_void_p * len(runs))(*[r.handle for r in runs])
    d = (ctypes.c_double * len(runs))(*dts)
    _check(_lib.vx_runs_advance(arr, d, len(runs)))


def calculate_dt_many(runs: list[SolverManager]) -> list[float]:
    """CalculateDt of several runs of one context in one launch."""
    arr = (ctypes.c_void_p * len(runs))(*[r.handle for r in runs])
    out = (ctypes.c_double * len(runs))()
    _check(_lib.vx_runs_calculate_dt(arr, out, len(runs)))
    return list(out)


class Server:
    """Continuous-batching serving loop on one context (vx_server)."""

    def __init__(self, ctx: Context, hbm_budget_bytes: int, max_live: int = 64):
        h = ctypes.c_void_p()
        _check(_lib.vx_server_create(ctx.handle, int(hbm_budget_bytes), int(max_live), ctypes.byref(h)))
        self.ctx = ctx
        self._h = h
        ctx._runs.add(self)  # closed with the context, before it

    def clock(self) -> float:
        v = ctypes.c_double()
        _check(_lib.vx_server_clock(self._h, ctypes.byref(v)))
        return float(v.value)

    def submit(self, problem: Problem, steps: int, arrival: float | None = None, state_path=None) -> int:
        rid = ctypes.c_int64()
        t = self.clock() if arrival is None else float(arrival)
        path = None if state_path is None else str(state_path).encode()
        _check(_lib.vx_server_submit(self._h, ctypes.byref(problem.to_c()), int(steps), t, path, ctypes.byref(rid)))
        return int(rid.value)

    def step(self) -> tuple[int, int]:
        live, waiting = ctypes.c_int(), ctypes.c_int()
        _check(_lib.vx_server_step(self._h, ctypes.byref(live), ctypes.byref(waiting)))
        return int(live.value), int(waiting.value)

    def result(self, rid: int) -> dict:
        r = _RequestResult()
        _check(_lib.vx_server_result(self._h, rid, ctypes.byref(r)))
        out = {k: getattr(r, k) for k, _ in r._fields_}
        out["error"] = r.error.decode()
        return out

    def cancel(self, rid: int) -> None:
        _check(_lib.vx_server_cancel(self._h, rid))

    def set_regrid(self, enable: bool = True, after_s: float = 0.0) -> None:
        """The reference driver's regrid rule for every solve (on by default)."""
        _check(_lib.vx_server_set_regrid(self._h, int(enable), float(after_s)))

    def close(self) -> None:
        if self._h:
            _check(_lib.vx_server_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def autotune_many(runs: list[SolverManager]) -> tuple[int, int]:
    """Picks the FCT tile shape (p x x) for these runs' launch set; returns it."""
    arr = (ctypes.c_void_p * len(runs))(*[r.handle for r in runs])
    tj, ti = ctypes.c_int(), ctypes.c_int()
    _check(_lib.vx_runs_autotune(arr, len(runs), ctypes.byref(tj), ctypes.byref(ti)))
    return int(tj.value), int(ti.value)
