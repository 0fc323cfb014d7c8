"""Ensembles of independent systems stepped together (nbody_ensemble_* in
include/nbody_gb300.h).

    ens = Ensemble(crossover=4096)
    sid = ens.add(n, dt=0.0035, eps2=40.0, theta2=0.25)    # mode by crossover
    ens.init_device(sid, "plummer", seed=7, params=[50.0, 1.0, 20.0])   # or ens.upload(sid, system)
    ens.step(50, graph_steps=10)
    system = ens.download(sid)

A system's trajectory does not depend on the other systems of the ensemble.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import (_INIT_KINDS, _MODES, INTEGRATOR_CPU, INTEGRATOR_GPU_EULER, KEYS_MORTON, KEYS_OCTREE, MODE_BH,
               MODE_PP, OK, NBodyError, ParticleSystem, _f, _i64, _ptr, lib)

PP_SHAPES = {"128x2": 0, "256x2": 1, "256x4": 2, "128x4": 3}


class Ensemble:
    def __init__(self, crossover: int = 4096, device: int = 0, pp_shape="256x2", key_mode="octree"):
        self._e = ctypes.c_void_p()
        self.crossover = int(crossover)
        self._check(lib().nbody_ensemble_create(ctypes.byref(self._e), int(device), self.crossover),
                    "nbody_ensemble_create")
        self.set_options(pp_shape, key_mode)

    def _check(self, rc: int, where: str) -> None:
        if rc != OK:
            detail = lib().nbody_ensemble_last_error(self._e).decode() if self._e else ""
            raise NBodyError(rc, where, detail)

    def set_options(self, pp_shape="256x2", key_mode="octree") -> None:
        shape = PP_SHAPES.get(pp_shape, pp_shape)
        keys = {"octree": KEYS_OCTREE, "morton": KEYS_MORTON}.get(key_mode, key_mode)
        self._check(lib().nbody_ensemble_set_options(self._e, int(shape), int(keys)), "nbody_ensemble_set_options")

    def set_stream(self, stream_ptr: int | None) -> None:
        self._check(lib().nbody_ensemble_set_stream(self._e, stream_ptr), "nbody_ensemble_set_stream")

    def add(self, n: int, dt: float, eps2: float, theta2: float = 0.25, mode=None, integrator="cpu") -> int:
        m = -1 if mode is None else _MODES[mode]
        integ = {"cpu": INTEGRATOR_CPU, "gpu_euler": INTEGRATOR_GPU_EULER}.get(integrator, integrator)
        sid = ctypes.c_int()
        self._check(lib().nbody_ensemble_add(self._e, int(n), float(dt), float(eps2), float(theta2), m, int(integ),
                                             ctypes.byref(sid)), "nbody_ensemble_add")
        return sid.value

    def remove(self, sid: int) -> None:
        self._check(lib().nbody_ensemble_remove(self._e, int(sid)), "nbody_ensemble_remove")

    def info(self, sid: int):
        """(mode 'pp' / 'bh', n)."""
        m, n = ctypes.c_int(), ctypes.c_int64()
        self._check(lib().nbody_ensemble_system_info(self._e, int(sid), ctypes.byref(m), ctypes.byref(n)),
                    "nbody_ensemble_system_info")
        return ("pp" if m.value == MODE_PP else "bh"), n.value

    def upload(self, sid: int, system: ParticleSystem) -> None:
        self._check(lib().nbody_ensemble_upload(self._e, int(sid), _ptr(system.positions), _ptr(system.velocities),
                                                _ptr(system.accelerations), _ptr(system.masses)),
                    "nbody_ensemble_upload")

    def init_device(self, sid: int, kind, seed: int = 12345, params=None) -> None:
        k = _INIT_KINDS.get(kind, kind)
        vals = [] if params is None else [float(x) for x in params]
        buf = (_f * len(vals))(*vals) if vals else None
        self._check(lib().nbody_ensemble_init_device(self._e, int(sid), int(k), ctypes.c_uint64(seed & (2**64 - 1)),
                                                     buf, len(vals)), "nbody_ensemble_init_device")

    def step(self, steps: int = 1, graph_steps: int = 0) -> None:
        self._check(lib().nbody_ensemble_step(self._e, int(steps), int(graph_steps)), "nbody_ensemble_step")

    def download(self, sid: int, system: ParticleSystem | None = None, masses: bool = True) -> ParticleSystem:
        if system is None:
            _, n = self.info(sid)
            z = np.zeros((n, 4), np.float32)
            system = ParticleSystem(z, z.copy(), np.zeros(n, np.float32), z.copy())
        self._check(lib().nbody_ensemble_download(self._e, int(sid), _ptr(system.positions), _ptr(system.velocities),
                                                  _ptr(system.accelerations),
                                                  _ptr(system.masses) if masses else None),
                    "nbody_ensemble_download")
        return system

    def sync(self) -> None:
        self._check(lib().nbody_ensemble_sync(self._e), "nbody_ensemble_sync")

    def counts(self) -> dict:
        s, l = ctypes.c_int(), ctypes.c_int()
        p, b = _i64(), _i64()
        self._check(lib().nbody_ensemble_counts(self._e, ctypes.byref(s), ctypes.byref(p), ctypes.byref(b),
                                                ctypes.byref(l)), "nbody_ensemble_counts")
        return {"systems": s.value, "pp_bodies": p.value, "bh_bodies": b.value, "launches_per_step": l.value}

    def profile_enable(self, on: bool = True) -> None:
        """Per-stage CUDA-event timing (steps then run without graphs)."""
        self._check(lib().nbody_ensemble_profile_enable(self._e, int(on)), "nbody_ensemble_profile_enable")

    def profile_read(self) -> dict:
        """{stage name: (milliseconds, launches)} since the last read."""
        k = lib().nbody_stage_count()
        ms = (ctypes.c_double * k)()
        cnt = (ctypes.c_int * k)()
        self._check(lib().nbody_ensemble_profile_read(self._e, ms, cnt, k), "nbody_ensemble_profile_read")
        return {lib().nbody_stage_name(i).decode(): (ms[i], cnt[i]) for i in range(k) if cnt[i]}

    @staticmethod
    def footprint(n: int, mode) -> int:
        return int(lib().nbody_ensemble_footprint(int(n), _MODES[mode]))

    def close(self) -> None:
        if self._e:
            lib().nbody_ensemble_destroy(self._e)
            self._e = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
