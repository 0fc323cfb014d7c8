"""Python binding of libnbody_gb300 (the sm_103a gravity solve) over its C ABI.

The classes mirror the reference's solver plugin interface, MarcVivas/N-body
``class ParticleSolver`` (include/ParticleSolver.h:8-15), and its
``ParticleSystem`` state layout (include/ParticleSystem.h:100-104), so that
parity tests read like the reference's own call sequence::

    system = ParticleSystem(positions, velocities, masses)      # vec4 arrays
    solver = ParticleSolverCUDA(time_step, squared_softening, n, mode="pp")
    solver.update_particle_positions(system)                     # one step
    solver.get_squared_softening(); solver.uses_gpu()            # -> False

Errors raise NBodyError carrying the C status code (the reference exits or
throws std::runtime_error instead). The library must be built
(``nbody_gb300.build.build()``); there is no fallback: without it, or without a CUDA
device, construction fails loudly.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libnbody_gb300.so")

OK, ERR_ARG, ERR_CUDA, ERR_NOMEM, ERR_CAPACITY, ERR_TIMEOUT, ERR_STATE = range(7)
MODE_PP, MODE_BH = 0, 1
KEYS_OCTREE, KEYS_MORTON = 0, 1
INTEGRATOR_CPU, INTEGRATOR_GPU_EULER = 0, 1
# Device-side initial conditions (nbody_init_device); 1..6 are the reference's -i numbers.
INIT_CUBE, INIT_GALAXY, INIT_SPHERE, INIT_BALL, INIT_CUBE_SURFACE = 1, 2, 4, 5, 6
INIT_PLUMMER, INIT_UNIFORM_BALL, INIT_TWO_DISCS = 16, 17, 18
INIT_MAX_PARAMS = 8
_INIT_KINDS = {"cube": INIT_CUBE, "galaxy": INIT_GALAXY, "sphere": INIT_SPHERE, "ball": INIT_BALL,
               "cube_surface": INIT_CUBE_SURFACE, "plummer": INIT_PLUMMER, "uniform_ball": INIT_UNIFORM_BALL,
               "two_discs": INIT_TWO_DISCS}
_MODES = {"pp": MODE_PP, "bh": MODE_BH, MODE_PP: MODE_PP, MODE_BH: MODE_BH}

_lib = None
_vp = ctypes.c_void_p
_i64 = ctypes.c_int64
_f = ctypes.c_float
_i = ctypes.c_int
_ip = ctypes.POINTER(ctypes.c_int)

# name -> (restype, argtypes): every entry point declared in include/nbody_gb300.h
SIGNATURES = {
    "nbody_status_string": (ctypes.c_char_p, [_i]),
    "nbody_last_error": (ctypes.c_char_p, [_vp]),
    "nbody_create": (_i, [ctypes.POINTER(_vp), _i, _i, _i64, _f, _f, _f]),
    "nbody_destroy": (_i, [_vp]),
    "nbody_set_stream": (_i, [_vp, _vp]),
    "nbody_get_squared_softening": (_f, [_vp]),
    "nbody_update_host": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _i]),
    "nbody_upload": (_i, [_vp, _vp, _vp, _vp, _vp]),
    "nbody_step": (_i, [_vp, _i]),
    "nbody_download": (_i, [_vp, _vp, _vp, _vp, _vp]),
    "nbody_sync": (_i, [_vp]),
    "nbody_host_in_place": (_i, [_vp, _i64, _i]),
    "nbody_device_state": (_i, [_vp, ctypes.POINTER(_vp), ctypes.POINTER(_vp), ctypes.POINTER(_vp)]),
    "nbody_pp_forces_device": (_i, [_vp, _vp, _vp, _i64]),
    "nbody_pp_step_device": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _i64]),
    "nbody_pp_config": (_i, [_vp, _i64, _ip, _ip, _ip]),
    "nbody_profile_enable": (_i, [_vp, _i]),
    "nbody_profile_read": (_i, [_vp, ctypes.POINTER(ctypes.c_double), _ip, _i]),
    "nbody_stage_name": (ctypes.c_char_p, [_i]),
    "nbody_stage_count": (_i, []),
    "nbody_pp_forces_noalloc": (_i, [_vp, _vp, _i64, _f, _vp, _ip]),
    "nbody_device_order": (_i, [_vp, ctypes.POINTER(_vp)]),
    "nbody_bh_keys_device": (_i, [_vp, _vp, _i64, _vp, _vp]),
    "nbody_sort_pairs_device": (_i, [_vp, _vp, _vp, _i64]),
    "nbody_bh_forces_device": (_i, [_vp, _vp, _vp, _i64]),
    "nbody_bh_tree_export": (_i, [_vp, _vp, _i64, ctypes.POINTER(_i64), _vp]),
    "nbody_bh_counters": (_i, [_vp, _i, ctypes.POINTER(_i64), ctypes.POINTER(_i64)]),
    "nbody_set_key_mode": (_i, [_vp, _i]),
    "nbody_diagnostics": (_i, [_vp, ctypes.POINTER(ctypes.c_double)]),
    "nbody_set_integrator": (_i, [_vp, _i]),
    "nbody_init_device": (_i, [_vp, _i, ctypes.c_uint64, ctypes.POINTER(_f), _i]),
    "nbody_download_masses": (_i, [_vp, _vp]),
    "nbody_selftest_wait": (_i, [_i, _i64, _ip, ctypes.POINTER(ctypes.c_double)]),
    "nbody_ensemble_create": (_i, [ctypes.POINTER(_vp), _i, _i64]),
    "nbody_ensemble_destroy": (_i, [_vp]),
    "nbody_ensemble_last_error": (ctypes.c_char_p, [_vp]),
    "nbody_ensemble_set_stream": (_i, [_vp, _vp]),
    "nbody_ensemble_set_options": (_i, [_vp, _i, _i]),
    "nbody_ensemble_add": (_i, [_vp, _i64, _f, _f, _f, _i, _i, _ip]),
    "nbody_ensemble_remove": (_i, [_vp, _i]),
    "nbody_ensemble_system_info": (_i, [_vp, _i, _ip, ctypes.POINTER(_i64)]),
    "nbody_ensemble_upload": (_i, [_vp, _i, _vp, _vp, _vp, _vp]),
    "nbody_ensemble_init_device": (_i, [_vp, _i, _i, ctypes.c_uint64, ctypes.POINTER(_f), _i]),
    "nbody_ensemble_step": (_i, [_vp, _i, _i]),
    "nbody_ensemble_download": (_i, [_vp, _i, _vp, _vp, _vp, _vp]),
    "nbody_ensemble_sync": (_i, [_vp]),
    "nbody_ensemble_counts": (_i, [_vp, _ip, ctypes.POINTER(_i64), ctypes.POINTER(_i64), _ip]),
    "nbody_ensemble_footprint": (_i64, [_i64, _i]),
    "nbody_ensemble_profile_enable": (_i, [_vp, _i]),
    "nbody_ensemble_profile_read": (_i, [_vp, ctypes.POINTER(ctypes.c_double), _ip, _i]),
}


class NBodyError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        msg = f"{where}: {status_string(status)} (status {status})"
        if detail:
            msg += f": {detail}"
        super().__init__(msg)


def lib():
    """Loads libnbody_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise NBodyError(ERR_STATE, "load", f"{LIB_PATH} missing; run nbody_gb300.build.build()")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def selftest_wait(limit_us: int = 50_000, device: int = 0):
    """Runs the bounded-wait self-test (nbody_selftest_wait): returns
    (kernel status, milliseconds waited); the status is ERR_TIMEOUT when the
    wait gave up as designed."""
    st = ctypes.c_int(-1)
    ms = ctypes.c_double(0.0)
    rc = lib().nbody_selftest_wait(int(device), int(limit_us), ctypes.byref(st), ctypes.byref(ms))
    if rc != OK:
        raise NBodyError(rc, "nbody_selftest_wait")
    return st.value, ms.value


def status_string(status: int) -> str:
    try:
        return lib().nbody_status_string(status).decode()
    except Exception:  # library missing: still give a name
        return {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "out of memory", 4: "capacity exceeded",
                5: "device wait timed out", 6: "call out of order"}.get(status, "unknown status")


def _ptr(a) -> int | None:
    """Address of a numpy array, a torch tensor, or an int; None passes NULL."""
    if a is None:
        return None
    if isinstance(a, int):
        return a
    if isinstance(a, np.ndarray):
        if not a.flags["C_CONTIGUOUS"]:
            raise ValueError("array must be C-contiguous")
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        if hasattr(a, "is_contiguous") and not a.is_contiguous():
            raise ValueError("tensor must be contiguous")
        return a.data_ptr()
    raise TypeError(f"cannot take the address of {type(a)}")


def _vec4(a, n: int, name: str) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float32)
    if a.shape != (n, 4):
        raise ValueError(f"{name} must have shape ({n}, 4), got {a.shape}")
    return a


class ParticleSystem:
    """Host state in the reference's ParticleSystem layout (include/ParticleSystem.h:100-104).

    positions, velocities, accelerations, forces: float32 (n, 4) vec4 arrays,
    positions with w = 0; masses: float32 (n, 4) with the mass in column 0.
    Arrays may be pinned (e.g. torch pin_memory().numpy()) for faster copies.
    """

    def __init__(self, positions, velocities=None, masses=None, accelerations=None):
        positions = np.asarray(positions, dtype=np.float32)
        n = positions.shape[0]
        if positions.shape[1] == 3:
            positions = np.concatenate([positions, np.zeros((n, 1), np.float32)], axis=1)
        self.n = n
        self.positions = _vec4(positions, n, "positions")
        self.velocities = _vec4(np.zeros((n, 4), np.float32) if velocities is None else velocities, n, "velocities")
        self.accelerations = _vec4(np.zeros((n, 4), np.float32) if accelerations is None else accelerations, n,
                                   "accelerations")
        m = np.ones(n, np.float32) if masses is None else np.asarray(masses, np.float32)
        if m.ndim == 1:
            m4 = np.zeros((n, 4), np.float32)
            m4[:, 0] = m
            m = m4
        self.masses = _vec4(m, n, "masses")
        self.forces = np.zeros((n, 4), np.float32)

    def size(self) -> int:
        return self.n


class ParticleSolverCUDA:
    """Drop-in for the reference's ParticleSolver subclasses (-v 2 / -v 6 semantics on the GPU).

    mode "pp" replaces ParticleSolverCPUParallel(timeStep, squaredSoftening)
    (include/ParticleSolverCPUParallel.h:9); mode "bh" replaces
    ParticleSolverBHutCPUParallel(timeStep, squaredSoftening, n)
    (include/ParticleSolverBHutCPUParallel.h:9). theta2 is the squared opening
    angle (reference default 0.25, src/Octree/Octree.cpp:15).
    """

    def __init__(self, time_step: float, squared_softening: float, n: int, mode="pp", theta2: float = 0.25,
                 device: int = 0):
        self.n = int(n)
        self.mode = _MODES[mode]
        self.time_step = float(time_step)
        self.theta2 = float(theta2)
        self._ctx = ctypes.c_void_p()
        rc = lib().nbody_create(ctypes.byref(self._ctx), int(device), self.mode, self.n, self.time_step,
                                float(squared_softening), self.theta2)
        if rc != OK:
            raise NBodyError(rc, "nbody_create")

    # --- ParticleSolver interface (include/ParticleSolver.h:12-14)
    def update_particle_positions(self, system: ParticleSystem, steps: int = 1) -> None:
        if system.n != self.n:
            raise NBodyError(ERR_ARG, "update_particle_positions", f"system has {system.n} bodies, solver {self.n}")
        self._check(lib().nbody_update_host(self._ctx, _ptr(system.positions), _ptr(system.velocities),
                                            _ptr(system.accelerations), _ptr(system.masses), _ptr(system.forces),
                                            int(steps)), "nbody_update_host")

    def get_squared_softening(self) -> float:
        return float(lib().nbody_get_squared_softening(self._ctx))

    def uses_gpu(self) -> bool:
        # Host arrays are valid after every call (the reference's usesGPU() == false contract).
        return False

    # --- resident mode and device entry points
    def upload(self, system: ParticleSystem) -> None:
        self._check(lib().nbody_upload(self._ctx, _ptr(system.positions), _ptr(system.velocities),
                                       _ptr(system.accelerations), _ptr(system.masses)), "nbody_upload")

    def step(self, steps: int = 1) -> None:
        self._check(lib().nbody_step(self._ctx, int(steps)), "nbody_step")

    def download(self, system: ParticleSystem, masses: bool = False) -> None:
        """Resident state into the host arrays; masses=True also fills the masses
        (needed after init_device, when the host never held them)."""
        self._check(lib().nbody_download(self._ctx, _ptr(system.positions), _ptr(system.velocities),
                                         _ptr(system.accelerations), _ptr(system.forces)), "nbody_download")
        if masses:
            self._check(lib().nbody_download_masses(self._ctx, _ptr(system.masses)), "nbody_download_masses")

    def sync(self) -> None:
        self._check(lib().nbody_sync(self._ctx), "nbody_sync")

    def set_stream(self, stream_ptr: int | None) -> None:
        self._check(lib().nbody_set_stream(self._ctx, stream_ptr), "nbody_set_stream")

    def device_state(self):
        p, v, a = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        self._check(lib().nbody_device_state(self._ctx, ctypes.byref(p), ctypes.byref(v), ctypes.byref(a)),
                    "nbody_device_state")
        return p.value, v.value, a.value

    def pp_forces_device(self, pos_mass, force, n: int | None = None) -> None:
        n = self.n if n is None else int(n)
        self._check(lib().nbody_pp_forces_device(self._ctx, _ptr(pos_mass), _ptr(force), n),
                    "nbody_pp_forces_device")

    def pp_step_device(self, pos_in, pos_out, vel, acc, force=None, n: int | None = None) -> None:
        n = self.n if n is None else int(n)
        self._check(lib().nbody_pp_step_device(self._ctx, _ptr(pos_in), _ptr(pos_out), _ptr(vel), _ptr(acc),
                                               _ptr(force), n), "nbody_pp_step_device")

    def pp_config(self, n: int | None = None):
        n = self.n if n is None else int(n)
        k, s, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self._check(lib().nbody_pp_config(self._ctx, n, ctypes.byref(k), ctypes.byref(s), ctypes.byref(c)),
                    "nbody_pp_config")
        return {"bodies_per_thread": k.value, "slices": s.value, "ctas": c.value}

    def profile_enable(self, on: bool = True) -> None:
        self._check(lib().nbody_profile_enable(self._ctx, int(on)), "nbody_profile_enable")

    def profile_read(self) -> dict:
        """{stage name: (milliseconds, launches)} since the last read, for stages that ran."""
        k = lib().nbody_stage_count()
        ms = (ctypes.c_double * k)()
        cnt = (ctypes.c_int * k)()
        self._check(lib().nbody_profile_read(self._ctx, ms, cnt, k), "nbody_profile_read")
        return {lib().nbody_stage_name(i).decode(): (ms[i], cnt[i]) for i in range(k) if cnt[i]}

    def device_order(self):
        p = ctypes.c_void_p()
        self._check(lib().nbody_device_order(self._ctx, ctypes.byref(p)), "nbody_device_order")
        return p.value

    def bh_keys_device(self, pos_mass, keys_out, box_out=None, n: int | None = None) -> None:
        n = self.n if n is None else int(n)
        self._check(lib().nbody_bh_keys_device(self._ctx, _ptr(pos_mass), n, _ptr(keys_out), _ptr(box_out)),
                    "nbody_bh_keys_device")

    def sort_pairs_device(self, keys, vals, n: int | None = None) -> None:
        n = self.n if n is None else int(n)
        self._check(lib().nbody_sort_pairs_device(self._ctx, _ptr(keys), _ptr(vals), n), "nbody_sort_pairs_device")

    def bh_forces_device(self, pos_mass, force, n: int | None = None) -> None:
        n = self.n if n is None else int(n)
        self._check(lib().nbody_bh_forces_device(self._ctx, _ptr(pos_mass), _ptr(force), n),
                    "nbody_bh_forces_device")

    def bh_tree(self):
        """Pre-order records of the last Barnes-Hut build and the root box.

        Returns (cm, meta, box): cm float32 (M, 4) centre of mass + mass;
        meta int32 (M, 4): side^2 bits (float, -1 for leaves), next, first
        body, leaf body count; box float32 (6,)."""
        count = ctypes.c_int64()
        self._check(lib().nbody_bh_tree_export(self._ctx, None, 0, ctypes.byref(count), None), "nbody_bh_tree_export")
        m = count.value
        rec = np.zeros((max(m, 1), 8), np.float32)
        box = np.zeros(6, np.float32)
        self._check(lib().nbody_bh_tree_export(self._ctx, _ptr(rec), m, ctypes.byref(count), _ptr(box)),
                    "nbody_bh_tree_export")
        rec = rec[:m]
        return rec[:, :4].copy(), rec[:, 4:].view(np.int32).copy(), box

    def diagnostics(self) -> dict:
        """FP64 kinetic/potential energy, linear and angular momentum of the resident state."""
        out = (ctypes.c_double * 8)()
        self._check(lib().nbody_diagnostics(self._ctx, out), "nbody_diagnostics")
        v = list(out)
        return {"kinetic": v[0], "potential": v[1], "energy": v[0] + v[1], "momentum": v[2:5],
                "angular_momentum": v[5:8]}

    def init_device(self, kind, seed: int = 12345, params=None) -> None:
        """Seeded initial conditions generated on the GPU in place of upload().

        kind: a name of _INIT_KINDS or an INIT_* number; params: up to
        INIT_MAX_PARAMS floats replacing the kind's defaults in order."""
        k = _INIT_KINDS.get(kind, kind)
        vals = [] if params is None else [float(x) for x in params]
        buf = (_f * max(len(vals), 1))(*vals) if vals else None
        self._check(lib().nbody_init_device(self._ctx, int(k), ctypes.c_uint64(seed & (2**64 - 1)), buf, len(vals)),
                    "nbody_init_device")

    def set_integrator(self, kind) -> None:
        """'cpu' (the reference's CPU order, default) or 'gpu_euler' (its GLSL semi-implicit Euler)."""
        k = {"cpu": INTEGRATOR_CPU, "gpu_euler": INTEGRATOR_GPU_EULER}.get(kind, kind)
        self._check(lib().nbody_set_integrator(self._ctx, int(k)), "nbody_set_integrator")

    def set_key_mode(self, mode) -> None:
        """'octree' (the reference's FP32 cell descent, default) or 'morton' (morton.glsl quantisation)."""
        m = {"octree": KEYS_OCTREE, "morton": KEYS_MORTON}.get(mode, mode)
        self._check(lib().nbody_set_key_mode(self._ctx, int(m)), "nbody_set_key_mode")

    def bh_counters(self, enable: bool):
        """(pair evaluations, warp record visits) since the last call; then counting on/off."""
        a, b = ctypes.c_int64(), ctypes.c_int64()
        self._check(lib().nbody_bh_counters(self._ctx, int(enable), ctypes.byref(a), ctypes.byref(b)),
                    "nbody_bh_counters")
        return a.value, b.value

    def close(self) -> None:
        if self._ctx:
            lib().nbody_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int, where: str) -> None:
        if rc != OK:
            detail = lib().nbody_last_error(self._ctx).decode() if self._ctx else ""
            raise NBodyError(rc, where, detail)


from .ensemble import Ensemble  # noqa: E402  (uses the names above)
