"""ctypes bindings for the CPU oracles. TEST INFRASTRUCTURE ONLY.

Two libraries are wrapped:

* ``_build/libnbody_oracle.so`` -- this project's C restatement of the
  reference's CPU solve (nbody_oracle.c, morton_oracle.c). It builds anywhere.
* ``_ref/libnbody_ref.so`` -- the reference's own CPU solver sources compiled
  headless (ref_harness.cpp + shim/). It exists only where the reference
  checkout was available at build time; ``ref_available()`` says whether it
  loaded.

Only tests/, ``__graft_entry__.smoke()`` and the CPU legs of bench.py import
this module: it is the checker and the CPU baseline, never the product.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libnbody_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libnbody_ref.so")

_f = ctypes.POINTER(ctypes.c_float)
_d = ctypes.POINTER(ctypes.c_double)
_u64 = ctypes.POINTER(ctypes.c_uint64)
_u32 = ctypes.POINTER(ctypes.c_uint32)
_i64 = ctypes.POINTER(ctypes.c_int64)
_port = None
_ref = None


def reference_dir() -> str | None:
    """The reference checkout: $NBODY_REFERENCE_DIR, else the Makefile's REF
    default; None when neither holds the reference's sources (as on hosts
    that carry only the fixtures)."""
    d = os.environ.get("NBODY_REFERENCE_DIR")
    if not d:
        r = subprocess.run(["make", "-s", "--no-print-directory", "-C", HERE, "print-ref"], capture_output=True,
                           text=True)
        d = r.stdout.strip() if r.returncode == 0 else ""
    return d if d and os.path.isdir(os.path.join(d, "src")) else None


def build(reference: bool = True) -> None:
    """Compile the port (always) and the reference build (when its sources exist)."""
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    ref_dir = reference_dir() if reference else None
    if ref_dir:
        subprocess.run(["make", "-s", "-j8", "-C", HERE, "ref", f"REF={ref_dir}"], check=True)


def _p(a, t=_f):
    return None if a is None else a.ctypes.data_as(t)


def port():
    global _port
    if _port is None:
        if not os.path.exists(PORT_SO):
            build(reference=False)
        lib = ctypes.CDLL(PORT_SO)
        lib.orc_bbox.argtypes = [ctypes.c_int64, _f, _f, _f]
        lib.orc_morton63.argtypes = [ctypes.c_int64, _f, _f, _f, _u64]
        lib.orc_octree_keys.argtypes = [ctypes.c_int64, _f, _f, _f, _u64]
        lib.orc_sort_stable.argtypes = [ctypes.c_int64, _u64, _u64, _u32]
        lib.orc_pp_forces.argtypes = [ctypes.c_int64, _f, _f, ctypes.c_float, _f, ctypes.c_int]
        lib.orc_integrate.argtypes = [ctypes.c_int64, _f, _f, _f, _f, ctypes.c_float, ctypes.c_int]
        lib.orc_pp_run.argtypes = [ctypes.c_int64, _f, _f, _f, _f, _f, ctypes.c_float, ctypes.c_float,
                                   ctypes.c_int, ctypes.c_int]
        lib.orc_pp_run.restype = ctypes.c_double
        lib.orc_bh_run.argtypes = [ctypes.c_int64, _f, _f, _f, _f, _f, ctypes.c_float, ctypes.c_float,
                                   ctypes.c_float, ctypes.c_int, ctypes.c_int, ctypes.c_int, _d, _f, _i64]
        lib.orc_direct_f64.argtypes = [ctypes.c_int64, _f, _f, ctypes.c_double, _i64, ctypes.c_int64, _d,
                                       ctypes.c_int]
        lib.orc_diagnostics_f64.argtypes = [ctypes.c_int64, _f, _f, _f, ctypes.c_double, _d, ctypes.c_int]
        _port = lib
    return _port


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def ref():
    global _ref
    if _ref is None:
        lib = ctypes.CDLL(REF_SO)
        lib.ref_run.argtypes = [ctypes.c_int, ctypes.c_int, _f, _f, _f, _f, ctypes.c_float, ctypes.c_float,
                                ctypes.c_float, ctypes.c_int, ctypes.c_int, _f, _f, _f, _f, _d, _f]
        lib.ref_lagrange.argtypes = [ctypes.c_float] * 3 + [_f, _f, _f, _f]
        lib.ref_dump_text.argtypes = [ctypes.c_int, _f, _f, _f, _f, ctypes.c_char_p, ctypes.c_long]
        lib.ref_dump_text.restype = ctypes.c_long
        lib.ref_load_text.argtypes = [ctypes.c_char_p, ctypes.c_int, _f, _f, _f, _f]
        _ref = lib
    return _ref


def _f4(a):
    return np.ascontiguousarray(a, dtype=np.float32).reshape(-1, 4)


# ----------------------------------------------------------------- port calls
def bbox(pos4):
    pos4 = _f4(pos4)
    mn = np.zeros(3, np.float32)
    mx = np.zeros(3, np.float32)
    port().orc_bbox(len(pos4), _p(pos4), _p(mn), _p(mx))
    return mn, mx


def morton63(pos4, bmin, bmax):
    pos4 = _f4(pos4)
    keys = np.zeros(len(pos4), np.uint64)
    port().orc_morton63(len(pos4), _p(pos4), _p(np.asarray(bmin, np.float32)), _p(np.asarray(bmax, np.float32)),
                        _p(keys, _u64))
    return keys


def octree_keys(pos4, bmin, bmax):
    pos4 = _f4(pos4)
    keys = np.zeros(len(pos4), np.uint64)
    port().orc_octree_keys(len(pos4), _p(pos4), _p(np.asarray(bmin, np.float32)), _p(np.asarray(bmax, np.float32)),
                           _p(keys, _u64))
    return keys


def sort_stable(keys):
    keys = np.ascontiguousarray(keys, np.uint64)
    ks = np.zeros_like(keys)
    perm = np.zeros(len(keys), np.uint32)
    rc = port().orc_sort_stable(len(keys), _p(keys, _u64), _p(ks, _u64), _p(perm, _u32))
    assert rc == 0
    return ks, perm


def pp_forces(pos4, mass, eps2, threads=0):
    pos4 = _f4(pos4)
    mass = np.ascontiguousarray(mass, np.float32)
    out = np.zeros_like(pos4)
    port().orc_pp_forces(len(mass), _p(pos4), _p(mass), eps2, _p(out), threads)
    return out


def pp_run(pos4, vel4, acc4, mass, dt, eps2, steps, threads=0):
    """`steps` x (-v 2 force + reference integrator); returns (pos, vel, acc, force, seconds)."""
    pos4, vel4, acc4 = _f4(pos4).copy(), _f4(vel4).copy(), _f4(acc4).copy()
    mass = np.ascontiguousarray(mass, np.float32)
    force = np.zeros_like(pos4)
    secs = port().orc_pp_run(len(mass), _p(pos4), _p(vel4), _p(acc4), _p(mass), _p(force), dt, eps2, steps,
                             threads)
    return pos4, vel4, acc4, force, secs


def bh_run(pos4, vel4, acc4, mass, dt, eps2, steps, theta2=0.25, threads=0, patched=False):
    """`steps` x -v 6 step; returns (pos, vel, acc, force, info dict)."""
    pos4, vel4, acc4 = _f4(pos4).copy(), _f4(vel4).copy(), _f4(acc4).copy()
    mass = np.ascontiguousarray(mass, np.float32)
    force = np.zeros_like(pos4)
    secs = ctypes.c_double()
    rm = ctypes.c_float()
    used = ctypes.c_int64()
    rc = port().orc_bh_run(len(mass), _p(pos4), _p(vel4), _p(acc4), _p(mass), _p(force), dt, eps2, theta2, steps,
                           threads, int(patched), ctypes.byref(secs), ctypes.byref(rm), ctypes.byref(used))
    return pos4, vel4, acc4, force, {"rc": rc, "seconds": secs.value, "root_mass": rm.value,
                                     "nodes": used.value}


def direct_f64(pos4, mass, eps2, idx=None, threads=0):
    pos4 = _f4(pos4)
    mass = np.ascontiguousarray(mass, np.float32)
    n = len(mass)
    if idx is None:
        k = n
        pidx = None
    else:
        idx = np.ascontiguousarray(idx, np.int64)
        k = len(idx)
        pidx = _p(idx, _i64)
    out = np.zeros((k, 3), np.float64)
    port().orc_direct_f64(n, _p(pos4), _p(mass), float(eps2), pidx, k, _p(out, _d), threads)
    return out


def diagnostics_f64(pos4, vel4, mass, eps2, threads=0):
    pos4, vel4 = _f4(pos4), _f4(vel4)
    mass = np.ascontiguousarray(mass, np.float32)
    out = np.zeros(8, np.float64)
    port().orc_diagnostics_f64(len(mass), _p(pos4), _p(vel4), _p(mass), float(eps2), _p(out, _d), threads)
    return out


# ------------------------------------------------------------ reference calls
def ref_run(version, pos4, vel4, acc4, mass, dt, eps2, steps, theta2=0.0, threads=0):
    """Run the reference's own solver -v `version` (1, 2, 5, 6) for `steps` steps."""
    pos4, vel4, acc4 = _f4(pos4), _f4(vel4), _f4(acc4)
    mass = np.ascontiguousarray(mass, np.float32)
    n = len(mass)
    po, vo, ao, fo = (np.zeros((n, 4), np.float32) for _ in range(4))
    secs = ctypes.c_double()
    rm = ctypes.c_float()
    rc = ref().ref_run(version, n, _p(pos4), _p(vel4), _p(acc4), _p(mass), dt, eps2, theta2, steps, threads,
                       _p(po), _p(vo), _p(ao), _p(fo), ctypes.byref(secs), ctypes.byref(rm))
    assert rc == 0
    return po, vo, ao, fo, {"seconds": secs.value, "root_mass": rm.value}


def ref_lagrange(world=(5.0, 5.0, 5.0)):
    pos, vel, acc = (np.zeros((3, 4), np.float32) for _ in range(3))
    mass = np.zeros(3, np.float32)
    ref().ref_lagrange(*[float(w) for w in world], _p(pos), _p(vel), _p(acc), _p(mass))
    return pos, vel, acc, mass


def ref_dump_text(pos4, vel4, acc4, mass) -> str:
    pos4, vel4, acc4 = _f4(pos4), _f4(vel4), _f4(acc4)
    mass = np.ascontiguousarray(mass, np.float32)
    n = len(mass)
    size = ref().ref_dump_text(n, _p(pos4), _p(vel4), _p(acc4), _p(mass), None, 0)
    buf = ctypes.create_string_buffer(size + 1)
    ref().ref_dump_text(n, _p(pos4), _p(vel4), _p(acc4), _p(mass), buf, size)
    return buf.raw[:size].decode()
