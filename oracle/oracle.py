"""ctypes wrapper of the CPU oracle (libgi_oracle.so) and of the reference's
own kernels (_ref/libgiref.so).

TEST INFRASTRUCTURE.  Only tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline legs import this module.  Arrays are numpy float32 (n, 4) for
bodies; pair tables and runs are passed as plain dicts / tuples so this
module does not depend on the product package.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libgi_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libgiref.so")

PARAM_FIELDS = ("GMassFeFe", "GMassFeSi", "GMassSiSi", "KFeFe", "KSiSi", "KFeSi", "KRFeFe",
                "KRSiSi", "KRFeSi", "KRMix", "ShellBreakFe", "ShellBreakSi", "ShellBreakFeSi1",
                "ShellBreakFeSi2", "MassFe", "MassSi")

SEP_REF_INT, SEP_SIGN = 0, 1
BRANCH_F32, BRANCH_F64 = 0, 1
FMA_ALL = 15


class Params(C.Structure):
    _fields_ = [(n, C.c_float) for n in PARAM_FIELDS]


class Run(C.Structure):
    _fields_ = [("offset", C.c_int), ("n", C.c_int), ("nfe", C.c_int), ("params", C.c_int),
                ("dt", C.c_float), ("dt_over_mass_fe", C.c_float),
                ("dt_over_mass_si", C.c_float), ("damp", C.c_float)]


_lib = None
_ref = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise RuntimeError(f"{LIB} not built; run __graft_entry__.build()")
        L = C.CDLL(LIB)
        P, I, F, D = C.c_void_p, C.c_int, C.c_float, C.c_double
        L.gio_version.restype = I
        L.gio_max_threads.restype = I
        L.gio_forces_ref.argtypes = [P, P, P, P, I, P, I, I, I]
        L.gio_forces_ref_subset.argtypes = [P, P, P, I, P, P, I, P, I, I, I]
        L.gio_move_ref.argtypes = [P, P, P, P, I, I, I]
        L.gio_forces_fp64.argtypes = [P, P, P, I, P, P, P, I, P, I, I, I]
        L.gio_potential_fp64.argtypes = [P, P, I, P, P, I, P, I]
        L.gio_diag_fp64.argtypes = [P, P, P, I, P, P, P]
        L.gio_count_flips.argtypes = [P, P, P, I, P, P, I, P, I, I]
        L.gio_integrate_fp64.argtypes = [P, P, I, I, P, D, I, I, P, I, I]
        L.gio_r2_threshold.argtypes = [F]
        L.gio_groups_ref.argtypes = [P, I, F, P]
        L.gio_groups_uf.argtypes = [P, I, F, P]
        L.gio_earth_moon_ref.argtypes = [P, I, P, P]
        L.gio_r2_threshold.restype = F
        _lib = L
    return _lib


def to_params(p) -> Params:
    """dict (or any object with the pair-table attributes) -> Params."""
    out = Params()
    for n in PARAM_FIELDS:
        setattr(out, n, float(p[n] if isinstance(p, dict) else getattr(p, n)))
    return out


def to_runs(runs) -> tuple:
    rs = []
    for r in runs:
        if isinstance(r, dict):
            rs.append(Run(r["offset"], r["n"], r["nfe"], r.get("params", 0), r.get("dt", 0.0),
                          r.get("dt_over_mass_fe", 0.0), r.get("dt_over_mass_si", 0.0),
                          r.get("damp", 0.0)))
        elif isinstance(r, (tuple, list)):
            rs.append(Run(*r))
        else:
            rs.append(Run(r.offset, r.n, r.nfe, r.params, r.dt, r.dt_over_mass_fe,
                          r.dt_over_mass_si, r.damp))
    arr = (Run * max(1, len(rs)))(*rs)
    return arr, len(rs)


def _params_arr(params):
    if not isinstance(params, (list, tuple)):
        params = [params]
    ps = [to_params(p) for p in params]
    return (Params * len(ps))(*ps)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def forces_ref(pos, vel, runs, params, sep_test=SEP_REF_INT, fma_mask=FMA_ALL, nthreads=0):
    pos, vel = _f32(pos), _f32(vel)
    force = np.zeros_like(pos)
    ra, nr = to_runs(runs)
    lib().gio_forces_ref(pos.ctypes.data, vel.ctypes.data, force.ctypes.data, ra, nr,
                         _params_arr(params), sep_test, fma_mask, nthreads)
    return force


def forces_ref_subset(pos, vel, idx, runs, params, sep_test=SEP_REF_INT, fma_mask=FMA_ALL,
                      nthreads=0):
    pos, vel = _f32(pos), _f32(vel)
    idx = np.ascontiguousarray(idx, dtype=np.int32)
    out = np.zeros((len(idx), 4), np.float32)
    ra, nr = to_runs(runs)
    lib().gio_forces_ref_subset(pos.ctypes.data, vel.ctypes.data, idx.ctypes.data, len(idx),
                                out.ctypes.data, ra, nr, _params_arr(params), sep_test, fma_mask,
                                nthreads)
    return out


def move_ref(pos, vel, force, runs, fma_mask=FMA_ALL, nthreads=0):
    pos, vel, force = _f32(pos).copy(), _f32(vel).copy(), _f32(force)
    ra, nr = to_runs(runs)
    lib().gio_move_ref(pos.ctypes.data, vel.ctypes.data, force.ctypes.data, ra, nr, fma_mask,
                       nthreads)
    return pos, vel


def forces_fp64(pos, vel, runs, params, idx=None, sep_test=SEP_REF_INT, branch=BRANCH_F32,
                nthreads=0):
    """Returns (force (k, 3) float64, sum_j |f_ij| (k,) float64)."""
    pos, vel = _f32(pos), _f32(vel)
    ra, nr = to_runs(runs)
    if idx is None:
        k = sum(ra[i].n for i in range(nr))
        ip = None
    else:
        idx = np.ascontiguousarray(idx, dtype=np.int32)
        k = len(idx)
        ip = idx.ctypes.data
    out = np.zeros((k, 3), np.float64)
    absf = np.zeros(k, np.float64)
    lib().gio_forces_fp64(pos.ctypes.data, vel.ctypes.data, ip, k, out.ctypes.data,
                          absf.ctypes.data, ra, nr, _params_arr(params), sep_test, branch, nthreads)
    return out, absf


def potential_fp64(pos, runs, params, idx=None, nthreads=0):
    pos = _f32(pos)
    ra, nr = to_runs(runs)
    if idx is None:
        k = sum(ra[i].n for i in range(nr))
        ip = None
    else:
        idx = np.ascontiguousarray(idx, dtype=np.int32)
        k = len(idx)
        ip = idx.ctypes.data
    out = np.zeros(k, np.float64)
    lib().gio_potential_fp64(pos.ctypes.data, ip, k, out.ctypes.data, ra, nr, _params_arr(params),
                             nthreads)
    return out


def diag_fp64(pos, vel, run, params, label=None, scope=0):
    pos, vel = _f32(pos), _f32(vel)
    ra, _ = to_runs([run])
    out = np.zeros(15, np.float64)
    lp = None
    if label is not None:
        label = np.ascontiguousarray(label, dtype=np.uint8)
        lp = label.ctypes.data
    lib().gio_diag_fp64(pos.ctypes.data, vel.ctypes.data, lp, scope, ra, _params_arr(params),
                        out.ctypes.data)
    return out


def count_flips(pos, vel, idx, runs, params, sep_test=SEP_REF_INT, nthreads=0):
    pos, vel = _f32(pos), _f32(vel)
    idx = np.ascontiguousarray(idx, dtype=np.int32)
    out = np.zeros(2, np.int64)
    ra, nr = to_runs(runs)
    lib().gio_count_flips(pos.ctypes.data, vel.ctypes.data, idx.ctypes.data, len(idx),
                          out.ctypes.data, ra, nr, _params_arr(params), sep_test, nthreads)
    return int(out[0]), int(out[1])


def integrate_fp64(pos, vel, nfe, params, dt, nsteps, every, sep_test=SEP_REF_INT, nthreads=0):
    """FP64 trajectory of one run (double state, double predicates).
    Returns (pos (n, 3) float64, vel (n, 3) float64, log (k, 7)) with log
    rows [E, Lx, Ly, Lz, Px, Py, Pz] at step 0 and every `every` steps."""
    X = np.ascontiguousarray(np.asarray(pos)[:, :3], dtype=np.float64).copy()
    V = np.ascontiguousarray(np.asarray(vel)[:, :3], dtype=np.float64).copy()
    nrec = (nsteps // every + 1) if every > 0 else 0
    log = np.zeros((max(nrec, 1), 7), np.float64)
    lib().gio_integrate_fp64(X.ctypes.data, V.ctypes.data, len(X), int(nfe),
                             _params_arr(params), float(dt), int(nsteps), int(every),
                             log.ctypes.data, sep_test, nthreads)
    return X, V, log[:nrec]


def material_params(G=1.0, D=1.0, mass_fe=1.0, mass_si=0.4, k_fe=5.0, k_si=1.5, kr_fe=0.02,
                    kr_si=0.01, sd_fe=0.002, sd_si=0.001) -> dict:
    """The pair table of loadKernalConstantStructures (impactAddTime.cu:128-170)
    for a general G and Si mass, computed in double and stored as float."""
    f = np.float32
    mix_fe_first = sd_fe >= sd_si
    return {
        "GMassFeFe": f(G * mass_fe * mass_fe), "GMassFeSi": f(G * mass_fe * mass_si),
        "GMassSiSi": f(G * mass_si * mass_si), "KFeFe": f(2.0 * k_fe), "KSiSi": f(2.0 * k_si),
        "KFeSi": f(k_fe + k_si), "KRFeFe": f(2.0 * k_fe * kr_fe), "KRSiSi": f(2.0 * k_si * kr_si),
        "KRFeSi": f(k_fe * kr_fe + k_si * kr_si),
        "KRMix": f(k_fe + k_si * kr_si) if mix_fe_first else f(k_fe * kr_fe + k_si),
        "ShellBreakFe": f(D - D * sd_fe), "ShellBreakSi": f(D - D * sd_si),
        "ShellBreakFeSi1": f(D - D * (sd_si if mix_fe_first else sd_fe)),
        "ShellBreakFeSi2": f(D - D * (sd_fe if mix_fe_first else sd_si)),
        "MassFe": f(mass_fe), "MassSi": f(mass_si)}


def r2_threshold(s: float) -> float:
    return float(lib().gio_r2_threshold(s))


def max_threads() -> int:
    return int(lib().gio_max_threads())


# --------------------------------------------------- reference kernels (GPU) --

def ref_lib():
    """The reference's own kernels (oracle/_ref/libgiref.so), or None."""
    global _ref
    if _ref is None and os.path.exists(REF_LIB):
        L = C.CDLL(REF_LIB)
        P, I, F = C.c_void_p, C.c_int, C.c_float
        for name in ("giref_forces_collision", "giref_forces_separate", "giref_move_collision"):
            getattr(L, name).argtypes = [P, P, P, P, I, P]
            getattr(L, name).restype = I
        L.giref_move_damped_separate.argtypes = [P, P, P, P, F, F, I, P]
        L.giref_move_damped_separate.restype = I
        L.giref_struct_sizes.argtypes = [P]
        _ref = L
    return _ref


REF_HOST_LIB = os.path.join(HERE, "_ref", "libgirefhost.so")
_ref_host = None


def ref_host_lib():
    """The reference's own host steps (oracle/_ref/libgirefhost.so, cut from
    its sources), or None."""
    global _ref_host
    if _ref_host is None and os.path.exists(REF_HOST_LIB):
        L = C.CDLL(REF_HOST_LIB)
        P, I, D = C.c_void_p, C.c_int, C.c_double
        L.giref_host_spin.argtypes = [P, P, P, D, D, D, D, I, P]
        L.giref_host_spin.restype = None
        L.giref_host_zero_drift.argtypes = [P, P, P, D, D, D, D]
        L.giref_host_zero_drift.restype = None
        L.giref_host_impact_setup.argtypes = [C.c_char_p, P, D, D, P, P]
        L.giref_host_impact_setup.restype = I
        _ref_host = L
    return _ref_host


def groups_ref(pos, touch=1.5):
    """Group number of every body, the reference's literal O(N^2) loop."""
    pos = _f32(pos)
    out = np.zeros(len(pos), np.int32)
    lib().gio_groups_ref(pos.ctypes.data, len(pos), touch, out.ctypes.data)
    return out


def groups_uf(pos, touch=1.5):
    """Group numbers by cell lists + union-find (larger N)."""
    pos = _f32(pos)
    out = np.zeros(len(pos), np.int32)
    lib().gio_groups_uf(pos.ctypes.data, len(pos), touch, out.ctypes.data)
    return out


def earth_moon_ref(group_id, bounds):
    """dict(earth, moon, n_earth, n_moon, n_groups, earth_counts, moon_counts)."""
    g = np.ascontiguousarray(group_id, dtype=np.int32)
    b = np.ascontiguousarray(bounds, dtype=np.int32)
    out = np.zeros(13, np.int32)
    lib().gio_earth_moon_ref(g.ctypes.data, len(g), b.ctypes.data, out.ctypes.data)
    return dict(earth=int(out[0]), moon=int(out[1]), n_earth=int(out[2]), n_moon=int(out[3]),
                n_groups=int(out[4]), earth_counts=[int(x) for x in out[5:9]],
                moon_counts=[int(x) for x in out[9:13]])
