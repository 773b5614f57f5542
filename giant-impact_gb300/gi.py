"""ctypes binding of libgi.so (include/gi_api.h) for Python callers.

Every call goes through the C ABI; there is no Python or CPU fallback.  If
libgi.so is missing or cannot run on this machine the calls raise GIError.
Device pointers are plain integers (e.g. torch.Tensor.data_ptr()), streams
are integers holding a cudaStream_t (0 = legacy default stream).
"""
from __future__ import annotations

import ctypes as C
import os
import re

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
LIB_PATH = os.path.join(PKG, "lib", "libgi.so")
HEADER = os.path.join(ROOT, "include", "gi_api.h")

GI_OK = 0
GI_SEP_REF_INT, GI_SEP_SIGN = 0, 1
GI_ACCUM_PAIRED, GI_ACCUM_FP32, GI_ACCUM_FP64, GI_ACCUM_KAHAN = 0, 1, 2, 3
STATUS = {0: "GI_OK", 1: "GI_ERR_INVALID_ARG", 2: "GI_ERR_BAD_SIZE", 3: "GI_ERR_ALIGNMENT",
          4: "GI_ERR_CUDA", 5: "GI_ERR_TIMEOUT", 6: "GI_ERR_NO_DEVICE", 7: "GI_ERR_OUT_OF_MEMORY",
          8: "GI_ERR_PARAMS", 9: "GI_ERR_IO", 10: "GI_ERR_FORMAT", 11: "GI_ERR_CAPACITY"}


class GIError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


class PairParams(C.Structure):
    _fields_ = [(n, C.c_float) for n in (
        "GMassFeFe", "GMassFeSi", "GMassSiSi", "KFeFe", "KSiSi", "KFeSi", "KRFeFe", "KRSiSi",
        "KRFeSi", "KRMix", "ShellBreakFe", "ShellBreakSi", "ShellBreakFeSi1", "ShellBreakFeSi2",
        "MassFe", "MassSi")]

    def as_dict(self) -> dict:
        return {n: getattr(self, n) for n, _ in self._fields_}


class Run(C.Structure):
    _fields_ = [("offset", C.c_int), ("n", C.c_int), ("nfe", C.c_int), ("params", C.c_int),
                ("dt", C.c_float), ("dt_over_mass_fe", C.c_float),
                ("dt_over_mass_si", C.c_float), ("damp", C.c_float)]


class Options(C.Structure):
    _fields_ = [("sep_test", C.c_int), ("accum", C.c_int), ("dense_min", C.c_int),
                ("cluster_tries", C.c_int)]


class Tuning(C.Structure):
    _fields_ = [("i_per_thread", C.c_int), ("jchunk", C.c_int)]


_FC = ["GMassFeFe", "GMassFeSi", "KFeFe", "KSiSi", "KFeSi", "KRFeFe", "KRSiSi", "KRFeSi",
       "KRMix", "ShellBreakFe", "ShellBreakSi", "ShellBreakFeSi1", "ShellBreakFeSi2"]


class ForceCollisionConsts(C.Structure):
    _fields_ = [(n, C.c_float) for n in _FC] + [("NFe", C.c_int)]


class MoveCollisionConsts(C.Structure):
    _fields_ = [("Dt", C.c_float), ("DtOverMassFe", C.c_float), ("DtOverMassSi", C.c_float),
                ("NFe", C.c_int)]


class ForceSeparateConsts(C.Structure):
    _fields_ = [(n, C.c_float) for n in _FC] + [("boarder1", C.c_int), ("boarder2", C.c_int),
                                                 ("boarder3", C.c_int)]


class MoveSeparateConsts(C.Structure):
    _fields_ = [("Dt", C.c_float), ("DtOverMassFe", C.c_float), ("DtOverMassSi", C.c_float),
                ("boarder1", C.c_int), ("boarder2", C.c_int), ("boarder3", C.c_int)]


class ServerConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_longlong), ("max_live_runs", C.c_int),
                ("steps_per_round", C.c_int), ("policy", C.c_int),
                ("fill_interactions", C.c_longlong)]


SERVE_SHARE, SERVE_SHORTEST = 0, 1


class RequestInfo(C.Structure):
    _fields_ = [("state", C.c_int), ("n", C.c_int), ("steps_done", C.c_int), ("nsteps", C.c_int),
                ("t_submit", C.c_double), ("t_admit", C.c_double), ("t_done", C.c_double),
                ("bytes", C.c_longlong)]


class ServerStats(C.Structure):
    _fields_ = [("live", C.c_int), ("queued", C.c_int), ("completed", C.c_longlong),
                ("rounds", C.c_longlong), ("bytes_in_use", C.c_longlong),
                ("pool_bodies", C.c_longlong), ("interactions", C.c_longlong),
                ("cancelled", C.c_longlong)]


class SetupGenerating(C.Structure):
    _fields_ = [("spin1", C.c_float * 4), ("spin2", C.c_float * 4),
                ("frac_earth_mass1", C.c_double), ("frac_earth_mass2", C.c_double),
                ("frac_fe1", C.c_double), ("frac_si1", C.c_double), ("frac_fe2", C.c_double),
                ("frac_si2", C.c_double), ("damp1", C.c_float), ("damp2", C.c_float),
                ("n", C.c_int), ("damp_time", C.c_double), ("damp_rest_time", C.c_double),
                ("spin_rest_time", C.c_double), ("dt", C.c_double), ("density_fe", C.c_double),
                ("density_si", C.c_double), ("k_fe", C.c_double), ("k_si", C.c_double),
                ("kr_fe", C.c_double), ("kr_si", C.c_double), ("sd_fe", C.c_double),
                ("sd_si", C.c_double), ("draw_rate", C.c_int)]


class SetupImpactInit(C.Structure):
    _fields_ = [("pos1", C.c_float * 3), ("pos2", C.c_float * 3), ("vel1", C.c_float * 3),
                ("vel2", C.c_float * 3)]


class SetupAddTime(C.Structure):
    _fields_ = [("additional_time_days", C.c_double), ("dt", C.c_double),
                ("draw_rate", C.c_int), ("record_rate", C.c_int), ("recenter_rate", C.c_int)]


class BodyParams(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "unit_time", "unit_length", "unit_mass", "mass_fe", "mass_si", "diameter", "k_fe", "k_si",
        "kr_fe", "kr_si", "sd_fe", "sd_si")] + [
        (n, C.c_int) for n in ("n", "nfe1", "nsi1", "nfe2", "nsi2")]


class GenerationPlan(C.Structure):
    _fields_ = [("body", BodyParams), ("mass_body1", C.c_double), ("mass_body2", C.c_double),
                ("damp_time", C.c_double), ("damp_rest_time", C.c_double),
                ("spin_rest_time", C.c_double), ("spin1_w", C.c_float), ("spin2_w", C.c_float),
                ("radius_of_earth", C.c_double)]


class EarthMoon(C.Structure):
    _fields_ = [("earth_label", C.c_int), ("moon_label", C.c_int), ("n_earth", C.c_int),
                ("n_moon", C.c_int), ("n_groups", C.c_int), ("earth_counts", C.c_int * 4),
                ("moon_counts", C.c_int * 4)]


class GenerateReport(C.Structure):
    _fields_ = [("steps", C.c_longlong), ("damped_steps", C.c_longlong),
                ("rest_steps", C.c_longlong), ("spin_steps", C.c_longlong),
                ("redraws", C.c_longlong), ("seconds", C.c_double)]


class View(C.Structure):
    _fields_ = [("eye", C.c_float * 3), ("center", C.c_float * 3), ("up", C.c_float * 3),
                ("frustum_half", C.c_float), ("near_plane", C.c_float), ("far_plane", C.c_float),
                ("width", C.c_int), ("height", C.c_int), ("point_size", C.c_int)]


def view(eye, center=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0), half=0.2, near=0.2, far=1200.0,
         width=1000, height=1000, point_size=2) -> "View":
    """The reference's camera by default (glFrustum(-0.2, 0.2, ...), 1000 px)."""
    return View((C.c_float * 3)(*eye), (C.c_float * 3)(*center), (C.c_float * 3)(*up), half, near,
                far, width, height, point_size)


class DiskInfo(C.Structure):
    _fields_ = [("n_disk", C.c_int), ("n_bound_inside", C.c_int), ("n_unbound", C.c_int),
                ("earth_mass", C.c_double), ("earth_radius", C.c_double)]


class AddTimeReport(C.Structure):
    _fields_ = [("steps", C.c_longlong), ("frames_written", C.c_longlong),
                ("recenters", C.c_longlong), ("start_time", C.c_double),
                ("end_time", C.c_double), ("seconds", C.c_double), ("earth_moon", EarthMoon),
                ("disk", DiskInfo), ("disk_stats", C.c_double * 15)]


SERVER_DRY_RUN = -1
REQ_QUEUED, REQ_LIVE, REQ_DONE = 0, 1, 2

_P = C.c_void_p
_SIGS = {
    "gi_version": ([], C.c_int),
    "gi_status_string": ([C.c_int], C.c_char_p),
    "gi_last_error": ([], C.c_char_p),
    "gi_device_info": ([C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                        C.POINTER(C.c_longlong)], C.c_int),
    "gi_forces_collision": ([_P, _P, _P, C.POINTER(ForceCollisionConsts), C.c_int, _P], C.c_int),
    "gi_forces_collision_noalloc": ([_P, _P, _P, C.POINTER(ForceCollisionConsts), C.c_int, _P],
                                    C.c_int),
    "gi_move_collision": ([_P, _P, _P, C.POINTER(MoveCollisionConsts), C.c_int, _P], C.c_int),
    "gi_forces_separate": ([_P, _P, _P, C.POINTER(ForceSeparateConsts), C.c_int, _P], C.c_int),
    "gi_move_damped_separate": ([_P, _P, _P, C.POINTER(MoveSeparateConsts), C.c_float,
                                 C.c_float, C.c_int, _P], C.c_int),
    "gi_ctx_create": ([C.POINTER(_P), C.c_int], C.c_int),
    "gi_ctx_destroy": ([_P], C.c_int),
    "gi_ctx_set_options": ([_P, C.POINTER(Options)], C.c_int),
    "gi_ctx_set_tuning": ([_P, C.POINTER(Tuning)], C.c_int),
    "gi_ctx_get_tuning": ([_P, C.c_int, C.POINTER(Tuning)], C.c_int),
    "gi_forces": ([_P, _P, _P, _P, C.POINTER(Run), C.c_int, C.POINTER(PairParams), C.c_int, _P],
                  C.c_int),
    "gi_autotune": ([_P, _P, _P, C.POINTER(Run), C.c_int, C.POINTER(PairParams), C.c_int, _P],
                    C.c_int),
    "gi_move": ([_P, _P, _P, _P, C.POINTER(Run), C.c_int, _P], C.c_int),
    "gi_step": ([_P, _P, _P, C.POINTER(Run), C.c_int, C.POINTER(PairParams), C.c_int, C.c_int,
                 _P], C.c_int),
    "gi_step_pingpong": ([_P, _P, _P, _P, _P, C.POINTER(Run), C.c_int, C.POINTER(PairParams),
                          C.c_int, C.c_int, _P], C.c_int),
    "gi_graph_create": ([_P, _P, _P, _P, _P, C.POINTER(Run), C.c_int, C.POINTER(PairParams),
                         C.c_int, C.c_int, _P, C.POINTER(_P)], C.c_int),
    "gi_graph_launch": ([_P, _P], C.c_int),
    "gi_graph_destroy": ([_P], C.c_int),
    "gi_diag_fp64": ([_P, _P, _P, _P, C.c_int, C.POINTER(Run), C.POINTER(PairParams),
                      C.POINTER(C.c_double), _P], C.c_int),
    "gi_potential_fp64": ([_P, _P, C.POINTER(Run), C.c_int, C.POINTER(PairParams), C.c_int,
                           C.POINTER(C.c_double), _P], C.c_int),
    "gi_run_host": ([_P, _P, _P, C.c_int, C.POINTER(Run), C.c_int, C.POINTER(PairParams),
                     C.c_int, C.c_int, _P], C.c_int),
    "gi_measure_ffma_peak": ([C.c_int, C.POINTER(C.c_double)], C.c_int),
    "gi_debug_fill_counters": ([_P, _P, C.c_uint], C.c_int),
    "gi_debug_pair_plan": ([_P, C.c_int, C.c_int, C.POINTER(C.c_longlong)], C.c_int),
    "gi_server_create": ([C.c_int, C.POINTER(ServerConfig), C.POINTER(PairParams), C.c_int,
                          C.POINTER(_P)], C.c_int),
    "gi_server_destroy": ([_P], C.c_int),
    "gi_server_submit": ([_P, _P, _P, C.POINTER(Run), C.c_int, C.POINTER(C.c_longlong)], C.c_int),
    "gi_server_round": ([_P, C.POINTER(C.c_int)], C.c_int),
    "gi_server_query": ([_P, C.c_longlong, C.POINTER(RequestInfo)], C.c_int),
    "gi_server_fetch": ([_P, C.c_longlong, _P, _P], C.c_int),
    "gi_server_get_stats": ([_P, C.POINTER(ServerStats)], C.c_int),
    "gi_server_cancel": ([_P, C.c_longlong], C.c_int),
    "gi_params_from_material": ([C.c_double] * 10 + [C.POINTER(PairParams)], C.c_int),
    "gi_params_from_collision_consts": ([C.POINTER(ForceCollisionConsts), C.POINTER(PairParams)],
                                        C.c_int),
    "gi_params_from_separate_consts": ([C.POINTER(ForceSeparateConsts), C.POINTER(PairParams)],
                                       C.c_int),
    "gi_read_setup_generating": ([C.c_char_p, C.POINTER(SetupGenerating)], C.c_int),
    "gi_read_setup_impact_init": ([C.c_char_p, C.POINTER(SetupImpactInit)], C.c_int),
    "gi_read_setup_add_time": ([C.c_char_p, C.POINTER(SetupAddTime)], C.c_int),
    "gi_read_body_params": ([C.c_char_p, C.POINTER(BodyParams)], C.c_int),
    "gi_write_body_params": ([C.c_char_p, C.POINTER(BodyParams)], C.c_int),
    "gi_read_view_centering": ([C.c_char_p, C.POINTER(C.c_float)], C.c_int),
    "gi_write_view_centering": ([C.c_char_p, C.POINTER(C.c_float)], C.c_int),
    "gi_derive_units": ([C.POINTER(SetupGenerating), C.POINTER(GenerationPlan)], C.c_int),
    "gi_collision_consts_from_body_params": ([C.POINTER(BodyParams), C.c_double,
                                              C.POINTER(ForceCollisionConsts),
                                              C.POINTER(MoveCollisionConsts)], C.c_int),
    "gi_separate_consts_from_body_params": ([C.POINTER(BodyParams), C.c_double,
                                             C.POINTER(ForceSeparateConsts),
                                             C.POINTER(MoveSeparateConsts)], C.c_int),
    "gi_write_body_file": ([C.c_char_p, _P, _P, C.c_int], C.c_int),
    "gi_read_body_file": ([C.c_char_p, _P, _P, C.c_int, C.POINTER(C.c_int)], C.c_int),
    "gi_frames_append": ([C.c_char_p, C.c_float, _P, _P, C.c_int], C.c_int),
    "gi_frames_count": ([C.c_char_p, C.c_int, C.POINTER(C.c_longlong)], C.c_int),
    "gi_frames_read": ([C.c_char_p, C.c_int, C.c_longlong, C.POINTER(C.c_float), _P, _P],
                       C.c_int),
    "gi_raw_bodies": ([C.c_ulonglong, C.POINTER(BodyParams), _P, _P, C.POINTER(C.c_longlong)],
                      C.c_int),
    "gi_spin_body": ([_P, _P, C.POINTER(GenerationPlan), C.c_int, C.POINTER(C.c_float),
                      C.c_float], C.c_int),
    "gi_zero_drift": ([_P, _P, C.POINTER(GenerationPlan)], C.c_int),
    "gi_write_target_impactor_stats": ([C.c_char_p, C.POINTER(GenerationPlan),
                                        C.POINTER(SetupGenerating), C.c_double, _P, _P], C.c_int),
    "gi_impact_initial_conditions": ([C.POINTER(BodyParams), C.POINTER(SetupImpactInit), _P, _P,
                                      _P, _P], C.c_int),
    "gi_system_stats_host": ([_P, _P, C.c_int, C.c_int, C.c_double, C.c_double,
                              C.POINTER(C.c_double)], C.c_int),
    "gi_write_initial_stats": ([C.c_char_p, C.POINTER(BodyParams), C.POINTER(C.c_double)],
                               C.c_int),
    "gi_find_earth_moon": ([_P, _P, C.c_int, C.c_float, C.POINTER(C.c_int), _P, _P,
                            C.POINTER(EarthMoon), _P], C.c_int),
    "gi_find_disk": ([_P, _P, _P, C.POINTER(Run), C.POINTER(PairParams), _P, C.POINTER(DiskInfo),
                      _P], C.c_int),
    "gi_view_basis": ([C.POINTER(View), C.POINTER(C.c_float)], C.c_int),
    "gi_splat": ([_P, _P, C.c_int, C.POINTER(C.c_int), C.POINTER(View), _P, _P], C.c_int),
    "gi_splat_scope": ([_P, _P, C.c_int, _P, C.POINTER(View), _P, _P], C.c_int),
    "gi_write_ppm": ([C.c_char_p, _P, C.c_int, C.c_int], C.c_int),
    "gi_render_frames": ([C.c_int, C.c_char_p, C.c_char_p, C.POINTER(View), C.c_int, C.c_char_p,
                          C.POINTER(C.c_longlong)], C.c_int),
    "gi_write_run_stats": ([C.c_char_p, C.POINTER(BodyParams), C.c_double, C.POINTER(EarthMoon),
                            C.POINTER(C.c_double)], C.c_int),
    "gi_generate_target_impactor": ([C.c_int, C.c_char_p, C.c_char_p, C.c_ulonglong,
                                     C.POINTER(GenerateReport)], C.c_int),
    "gi_impact_initialize": ([C.c_char_p, C.c_char_p, C.c_char_p], C.c_int),
    "gi_impact_add_time": ([C.c_int, C.c_char_p, C.c_char_p, C.c_char_p,
                            C.POINTER(AddTimeReport)], C.c_int),
    "gi_ic_uniform_ball": ([C.c_ulonglong, C.c_int, C.c_double, C.c_double, C.c_float, C.c_float,
                            C.c_float, C.c_float, _P, _P, C.POINTER(C.c_int)], C.c_int),
    "gi_ic_lattice": ([C.c_ulonglong, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int,
                       C.c_float, C.c_float, _P, _P], C.c_int),
}

_lib = None


def lib() -> C.CDLL:
    """Load libgi.so (built by __graft_entry__.build()); raise if absent."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise GIError(6, f"{LIB_PATH} is not built; run __graft_entry__.build()")
        L = C.CDLL(LIB_PATH)
        for name, (args, res) in _SIGS.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


def header_symbols() -> list[str]:
    """Names of every function declared in include/gi_api.h."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gi_[a-z0-9_]+)\s*\(", text)))


def check(status: int) -> None:
    if status != GI_OK:
        raise GIError(status, lib().gi_last_error().decode(errors="replace"))


def _arr(structs, cls):
    if isinstance(structs, cls):
        structs = [structs]
    structs = list(structs)
    a = (cls * max(1, len(structs)))(*structs)
    return a, len(structs)


def pair_plan(n: int, pcl: int = -1, ctx=None) -> dict:
    """The paired far field's decomposition of a run of n bodies with 2^pcl
    j-chunks per item (pcl < 0: ctx's choice, or the default one): host
    arithmetic only, usable without a GPU."""
    out = (C.c_longlong * 6)()
    check(lib().gi_debug_pair_plan(ctx.h if ctx is not None else None, n, pcl, out))
    return {"pcl": out[0], "chunks": out[1], "iblocks": out[2], "items": out[3],
            "stride": out[4], "items_block0": out[5]}


def params_from_material(G=1.0, diameter=1.0, mass_fe=1.0, mass_si=0.4, k_fe=5.0, k_si=1.5,
                         kr_fe=0.02, kr_si=0.01, sd_fe=0.002, sd_si=0.001) -> PairParams:
    p = PairParams()
    check(lib().gi_params_from_material(G, diameter, mass_fe, mass_si, k_fe, k_si, kr_fe, kr_si,
                                        sd_fe, sd_si, C.byref(p)))
    return p


def params_from_collision_consts(c: ForceCollisionConsts) -> PairParams:
    p = PairParams()
    check(lib().gi_params_from_collision_consts(C.byref(c), C.byref(p)))
    return p


def collision_consts(p: PairParams, nfe: int) -> ForceCollisionConsts:
    """Reference force struct from a pair table (the table's Si-Si gravity
    must be 1, as the reference kernel assumes)."""
    c = ForceCollisionConsts()
    for n in _FC:
        setattr(c, n, getattr(p, n))
    c.NFe = nfe
    return c


def separate_consts(p: PairParams, b1: int, b2: int, b3: int) -> ForceSeparateConsts:
    c = ForceSeparateConsts()
    for n in _FC:
        setattr(c, n, getattr(p, n))
    c.boarder1, c.boarder2, c.boarder3 = b1, b2, b3
    return c


def device_info(device: int = 0) -> dict:
    sm, ma, mi, mem = C.c_int(), C.c_int(), C.c_int(), C.c_longlong()
    check(lib().gi_device_info(device, C.byref(sm), C.byref(ma), C.byref(mi), C.byref(mem)))
    return {"sm_count": sm.value, "cc": (ma.value, mi.value), "mem_bytes": mem.value}


def measure_ffma_peak(device: int = 0) -> float:
    t = C.c_double()
    check(lib().gi_measure_ffma_peak(device, C.byref(t)))
    return t.value


def forces_collision(pos, vel, force, consts, n, stream=0):
    check(lib().gi_forces_collision(pos, vel, force, C.byref(consts), n, stream))


def forces_collision_noalloc(pos, vel, force, consts, n, stream=0):
    """gi_forces_collision without any device allocation (static scratch,
    n <= NOALLOC_MAX_BODIES; calls must not overlap on the GPU)."""
    check(lib().gi_forces_collision_noalloc(pos, vel, force, C.byref(consts), n, stream))


NOALLOC_MAX_BODIES = 32768


def move_collision(pos, vel, force, consts, n, stream=0):
    check(lib().gi_move_collision(pos, vel, force, C.byref(consts), n, stream))


def forces_separate(pos, vel, force, consts, n, stream=0):
    check(lib().gi_forces_separate(pos, vel, force, C.byref(consts), n, stream))


def move_damped_separate(pos, vel, force, consts, damp1, damp2, n, stream=0):
    check(lib().gi_move_damped_separate(pos, vel, force, C.byref(consts), damp1, damp2, n, stream))


class Context:
    """Owns a gi_ctx (scratch, options, tuning) on one device."""

    def __init__(self, device: int = 0, sep_test: int = GI_SEP_REF_INT,
                 accum: int = GI_ACCUM_PAIRED, dense_min: int = 0, cluster_tries: int = 0):
        h = C.c_void_p()
        check(lib().gi_ctx_create(C.byref(h), device))
        self.h = h
        self.set_options(sep_test, accum, dense_min, cluster_tries)

    def close(self):
        if self.h:
            lib().gi_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_options(self, sep_test=GI_SEP_REF_INT, accum=GI_ACCUM_PAIRED, dense_min=0,
                    cluster_tries=0):
        o = Options(sep_test, accum, dense_min, cluster_tries)
        check(lib().gi_ctx_set_options(self.h, C.byref(o)))

    def fill_counters(self, value: int, stream=0):
        """Test hook: overwrite the work-queue counters and split tickets of
        this stream's scratch with a memset byte pattern."""
        check(lib().gi_debug_fill_counters(self.h, stream, value))

    def set_tuning(self, i_per_thread=None, jchunk=0):
        if i_per_thread is None:
            check(lib().gi_ctx_set_tuning(self.h, None))
        else:
            t = Tuning(i_per_thread, jchunk)
            check(lib().gi_ctx_set_tuning(self.h, C.byref(t)))

    def get_tuning(self, n: int) -> tuple[int, int]:
        t = Tuning()
        check(lib().gi_ctx_get_tuning(self.h, n, C.byref(t)))
        return t.i_per_thread, t.jchunk

    def autotune(self, pos, vel, runs, params, stream=0):
        ra, nr = _arr(runs, Run)
        pa, npar = _arr(params, PairParams)
        check(lib().gi_autotune(self.h, pos, vel, ra, nr, pa, npar, stream))

    def forces(self, pos, vel, force, runs, params, stream=0):
        ra, nr = _arr(runs, Run)
        pa, npar = _arr(params, PairParams)
        check(lib().gi_forces(self.h, pos, vel, force, ra, nr, pa, npar, stream))

    def move(self, pos, vel, force, runs, stream=0):
        ra, nr = _arr(runs, Run)
        check(lib().gi_move(self.h, pos, vel, force, ra, nr, stream))

    def step(self, pos, vel, runs, params, nsteps, stream=0):
        ra, nr = _arr(runs, Run)
        pa, npar = _arr(params, PairParams)
        check(lib().gi_step(self.h, pos, vel, ra, nr, pa, npar, nsteps, stream))

    def step_pingpong(self, pos_a, vel_a, pos_b, vel_b, runs, params, nsteps, stream=0):
        ra, nr = _arr(runs, Run)
        pa, npar = _arr(params, PairParams)
        check(lib().gi_step_pingpong(self.h, pos_a, vel_a, pos_b, vel_b, ra, nr, pa, npar, nsteps,
                                     stream))

    def graph(self, pos_a, vel_a, pos_b, vel_b, runs, params, nsteps, stream):
        """Capture nsteps fused steps into a StepGraph (stream must not be 0)."""
        ra, nr = _arr(runs, Run)
        pa, npar = _arr(params, PairParams)
        h = C.c_void_p()
        check(lib().gi_graph_create(self.h, pos_a, vel_a, pos_b, vel_b, ra, nr, pa, npar, nsteps,
                                    stream, C.byref(h)))
        return StepGraph(h)

    def diag(self, pos, vel, run, params, label=None, scope=0, stream=0) -> list[float]:
        out = (C.c_double * 15)()
        check(lib().gi_diag_fp64(self.h, pos, vel, label, scope, C.byref(run), C.byref(params),
                                 out, stream))
        return list(out)

    def potential(self, pos, runs, params, stream=0) -> list[float]:
        ra, nr = _arr(runs, Run)
        pa, npar = _arr(params, PairParams)
        out = (C.c_double * max(1, nr))()
        check(lib().gi_potential_fp64(self.h, pos, ra, nr, pa, npar, out, stream))
        return list(out[:nr])

    def run_host(self, pos_host, vel_host, ntotal, runs, params, nsteps, stream=0):
        ra, nr = _arr(runs, Run)
        pa, npar = _arr(params, PairParams)
        check(lib().gi_run_host(self.h, pos_host, vel_host, ntotal, ra, nr, pa, npar, nsteps,
                                stream))


class StepGraph:
    """A captured step loop (gi_graph); launch() advances every run."""

    def __init__(self, h):
        self.h = h

    def launch(self, stream):
        check(lib().gi_graph_launch(self.h, stream))

    def close(self):
        if self.h:
            lib().gi_graph_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous-batching serving loop (gi_server_*)."""

    def __init__(self, params, device=0, budget_bytes=150 << 30, max_live_runs=64,
                 steps_per_round=100, policy=SERVE_SHARE, fill_interactions=0):
        pa, npar = _arr(params, PairParams)
        cfg = ServerConfig(budget_bytes, max_live_runs, steps_per_round, policy, fill_interactions)
        h = C.c_void_p()
        check(lib().gi_server_create(device, C.byref(cfg), pa, npar, C.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            lib().gi_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, pos, vel, run, nsteps) -> int:
        import numpy as np
        pos = np.ascontiguousarray(pos, np.float32)
        vel = np.ascontiguousarray(vel, np.float32)
        rid = C.c_longlong()
        check(lib().gi_server_submit(self.h, pos.ctypes.data, vel.ctypes.data, C.byref(run), nsteps,
                                     C.byref(rid)))
        return rid.value

    def round(self) -> int:
        n = C.c_int()
        check(lib().gi_server_round(self.h, C.byref(n)))
        return n.value

    def query(self, rid) -> RequestInfo:
        info = RequestInfo()
        check(lib().gi_server_query(self.h, rid, C.byref(info)))
        return info

    def fetch(self, rid, n):
        import numpy as np
        pos = np.zeros((n, 4), np.float32)
        vel = np.zeros((n, 4), np.float32)
        check(lib().gi_server_fetch(self.h, rid, pos.ctypes.data, vel.ctypes.data))
        return pos, vel

    def cancel(self, rid):
        check(lib().gi_server_cancel(self.h, rid))

    def stats(self) -> ServerStats:
        st = ServerStats()
        check(lib().gi_server_get_stats(self.h, C.byref(st)))
        return st


def ic_uniform_ball(seed, n, radius=20.0, fe_fraction=0.3, mass_fe=1.0, mass_si=0.4,
                    tag_fe=0.0, tag_si=1.0):
    """Returns (pos, vel, nfe) as numpy float32 arrays of shape (n, 4)."""
    import numpy as np
    pos = np.zeros((n, 4), np.float32)
    vel = np.zeros((n, 4), np.float32)
    nfe = C.c_int()
    check(lib().gi_ic_uniform_ball(seed, n, radius, fe_fraction, mass_fe, mass_si, tag_fe, tag_si,
                                   pos.ctypes.data, vel.ctypes.data, C.byref(nfe)))
    return pos, vel, nfe.value


def ic_lattice(seed, n, spacing=0.999, jitter=0.004, vel_sigma=1.0, nfe=None, mass_fe=1.0,
               mass_si=0.4):
    import numpy as np
    if nfe is None:
        nfe = n // 3
    pos = np.zeros((n, 4), np.float32)
    vel = np.zeros((n, 4), np.float32)
    check(lib().gi_ic_lattice(seed, n, spacing, jitter, vel_sigma, nfe, mass_fe, mass_si,
                              pos.ctypes.data, vel.ctypes.data))
    return pos, vel, nfe


# ------------------------------------------------------------------ files --

def _b(path) -> bytes:
    return os.fsencode(path)


def _f4(a, n=None):
    """Contiguous float32 (n, 4) array and its address."""
    import numpy as np
    a = np.ascontiguousarray(a, dtype=np.float32)
    if n is not None and a.shape != (n, 4):
        raise ValueError(f"expected shape ({n}, 4), got {a.shape}")
    return a, a.ctypes.data


def read_setup_generating(path) -> SetupGenerating:
    o = SetupGenerating()
    check(lib().gi_read_setup_generating(_b(path), C.byref(o)))
    return o


def read_setup_impact_init(path) -> SetupImpactInit:
    o = SetupImpactInit()
    check(lib().gi_read_setup_impact_init(_b(path), C.byref(o)))
    return o


def read_setup_add_time(path) -> SetupAddTime:
    o = SetupAddTime()
    check(lib().gi_read_setup_add_time(_b(path), C.byref(o)))
    return o


def read_body_params(path) -> BodyParams:
    o = BodyParams()
    check(lib().gi_read_body_params(_b(path), C.byref(o)))
    return o


def write_body_params(path, b: BodyParams) -> None:
    check(lib().gi_write_body_params(_b(path), C.byref(b)))


def read_view_centering(path) -> list[float]:
    v = (C.c_float * 6)()
    check(lib().gi_read_view_centering(_b(path), v))
    return list(v)


def write_view_centering(path, v) -> None:
    a = (C.c_float * 6)(*v)
    check(lib().gi_write_view_centering(_b(path), a))


def derive_units(setup: SetupGenerating) -> GenerationPlan:
    o = GenerationPlan()
    check(lib().gi_derive_units(C.byref(setup), C.byref(o)))
    return o


def collision_consts_from_body_params(b: BodyParams, dt: float):
    fc, mc = ForceCollisionConsts(), MoveCollisionConsts()
    check(lib().gi_collision_consts_from_body_params(C.byref(b), dt, C.byref(fc), C.byref(mc)))
    return fc, mc


def separate_consts_from_body_params(b: BodyParams, dt: float):
    fc, mc = ForceSeparateConsts(), MoveSeparateConsts()
    check(lib().gi_separate_consts_from_body_params(C.byref(b), dt, C.byref(fc), C.byref(mc)))
    return fc, mc


def params_from_separate_consts(c: ForceSeparateConsts) -> PairParams:
    p = PairParams()
    check(lib().gi_params_from_separate_consts(C.byref(c), C.byref(p)))
    return p


def write_body_file(path, pos, vel) -> None:
    pa, pp = _f4(pos)
    va, vp = _f4(vel, len(pa))
    check(lib().gi_write_body_file(_b(path), pp, vp, len(pa)))


def read_body_file(path):
    import numpy as np
    n = C.c_int()
    check(lib().gi_read_body_file(_b(path), None, None, 0, C.byref(n)))
    pos = np.zeros((n.value, 4), np.float32)
    vel = np.zeros((n.value, 4), np.float32)
    check(lib().gi_read_body_file(_b(path), pos.ctypes.data, vel.ctypes.data, n.value,
                                  C.byref(n)))
    return pos, vel


def frames_append(path, time, pos, vel) -> None:
    pa, pp = _f4(pos)
    va, vp = _f4(vel, len(pa))
    check(lib().gi_frames_append(_b(path), time, pp, vp, len(pa)))


def frames_count(path, n) -> int:
    k = C.c_longlong()
    check(lib().gi_frames_count(_b(path), n, C.byref(k)))
    return k.value


def frames_read(path, n, frame=-1):
    import numpy as np
    t = C.c_float()
    pos = np.zeros((n, 4), np.float32)
    vel = np.zeros((n, 4), np.float32)
    check(lib().gi_frames_read(_b(path), n, frame, C.byref(t), pos.ctypes.data, vel.ctypes.data))
    return t.value, pos, vel


def raw_bodies(seed, b: BodyParams):
    """Returns (pos, vel, redraws) in the builder order [Fe1, Si1, Fe2, Si2]."""
    import numpy as np
    pos = np.zeros((b.n, 4), np.float32)
    vel = np.zeros((b.n, 4), np.float32)
    r = C.c_longlong()
    check(lib().gi_raw_bodies(seed, C.byref(b), pos.ctypes.data, vel.ctypes.data, C.byref(r)))
    return pos, vel, r.value


def spin_body(pos, vel, plan: GenerationPlan, body, axis, w) -> None:
    """In place on float32 (n, 4) numpy arrays."""
    a = (C.c_float * 3)(*axis)
    check(lib().gi_spin_body(pos.ctypes.data, vel.ctypes.data, C.byref(plan), body, a, w))


def zero_drift(pos, vel, plan: GenerationPlan) -> None:
    check(lib().gi_zero_drift(pos.ctypes.data, vel.ctypes.data, C.byref(plan)))


def write_target_impactor_stats(path, plan, setup, dt, pos, vel) -> None:
    pa, pp = _f4(pos)
    va, vp = _f4(vel, len(pa))
    check(lib().gi_write_target_impactor_stats(_b(path), C.byref(plan), C.byref(setup), dt, pp,
                                               vp))


def impact_initial_conditions(b: BodyParams, s: SetupImpactInit, pos, vel):
    import numpy as np
    pa, pp = _f4(pos, b.n)
    va, vp = _f4(vel, b.n)
    po = np.zeros((b.n, 4), np.float32)
    vo = np.zeros((b.n, 4), np.float32)
    check(lib().gi_impact_initial_conditions(C.byref(b), C.byref(s), pp, vp, po.ctypes.data,
                                             vo.ctypes.data))
    return po, vo


def system_stats_host(pos, vel, nfe, mass_fe, mass_si) -> list[float]:
    pa, pp = _f4(pos)
    va, vp = _f4(vel, len(pa))
    out = (C.c_double * 10)()
    check(lib().gi_system_stats_host(pp, vp, len(pa), nfe, mass_fe, mass_si, out))
    return list(out)


def write_initial_stats(path, b: BodyParams, stats) -> None:
    a = (C.c_double * 10)(*stats)
    check(lib().gi_write_initial_stats(_b(path), C.byref(b), a))


def find_earth_moon(ctx: "Context", pos, n, touch, bounds, group=None, scope=None,
                    stream=0) -> EarthMoon:
    """pos, group, scope: device pointers (group/scope may be None)."""
    em = EarthMoon()
    bd = (C.c_int * 3)(*bounds)
    check(lib().gi_find_earth_moon(ctx.h, pos, n, touch, bd, group, scope, C.byref(em), stream))
    return em


def find_disk(ctx: "Context", pos, vel, run: Run, params: PairParams, scope, stream=0) -> DiskInfo:
    """pos, vel, scope: device pointers; scope holds gi_find_earth_moon's labels
    and receives 3 for disk bodies."""
    d = DiskInfo()
    check(lib().gi_find_disk(ctx.h, pos, vel, C.byref(run), C.byref(params), scope, C.byref(d),
                             stream))
    return d


def write_run_stats(path, b: BodyParams, time, em: EarthMoon, scope_stats) -> None:
    flat = [float(x) for row in scope_stats for x in (list(row) + [0.0] * 15)[:15]]
    a = (C.c_double * 60)(*flat)
    check(lib().gi_write_run_stats(_b(path), C.byref(b), time, C.byref(em), a))


def generate_target_impactor(setup_path, info_dir, seed=1, device=0) -> GenerateReport:
    r = GenerateReport()
    check(lib().gi_generate_target_impactor(device, _b(setup_path), _b(info_dir), seed,
                                            C.byref(r)))
    return r


def impact_initialize(info_dir, setup_path, impact_info_dir) -> None:
    check(lib().gi_impact_initialize(_b(info_dir), _b(setup_path), _b(impact_info_dir)))


def impact_add_time(info_dir, setup_path, impact_dir, device=0) -> AddTimeReport:
    r = AddTimeReport()
    check(lib().gi_impact_add_time(device, _b(info_dir), _b(setup_path), _b(impact_dir),
                                   C.byref(r)))
    return r


# ---------------------------------------------------------------- pictures --

def view_basis(v: View) -> list[float]:
    out = (C.c_float * 12)()
    check(lib().gi_view_basis(C.byref(v), out))
    return list(out)


def splat(ctx: "Context", pos, n, bounds, v: View, stream=0):
    """pos: device pointer.  Returns a (height, width, 3) uint8 numpy image."""
    import numpy as np
    img = np.zeros((v.height, v.width, 3), np.uint8)
    bd = (C.c_int * 3)(*bounds)
    check(lib().gi_splat(ctx.h, pos, n, bd, C.byref(v), img.ctypes.data, stream))
    return img


def splat_scope(ctx: "Context", pos, n, scope, v: View, stream=0):
    """The analysis picture: only Earth (scope 1, blue) and Moon (scope 2,
    white) elements.  pos, scope: device pointers (scope: n bytes, as
    find_earth_moon writes them).  Returns a (height, width, 3) uint8 image."""
    import numpy as np
    img = np.zeros((v.height, v.width, 3), np.uint8)
    check(lib().gi_splat_scope(ctx.h, pos, n, scope, C.byref(v), img.ctypes.data, stream))
    return img


def write_ppm(path, img) -> None:
    import numpy as np
    img = np.ascontiguousarray(img, dtype=np.uint8)
    check(lib().gi_write_ppm(_b(path), img.ctypes.data, img.shape[1], img.shape[0]))


def render_frames(info_dir, frames_path, v: View, out_prefix, every=1, device=0) -> int:
    k = C.c_longlong()
    check(lib().gi_render_frames(device, _b(info_dir), _b(frames_path), C.byref(v), every,
                                 _b(out_prefix), C.byref(k)))
    return k.value
