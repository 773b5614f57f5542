"""CPU tests of the reference file formats and the host steps of building
bodies and setting up an impact (gi_formats.cpp), against the restatement in
oracle/formats_oracle.py.  Where the reference sources are present, the text
files the library writes are also checked line by line against the
reference writers' own fprintf formats."""
from __future__ import annotations

import ctypes as C
import hashlib
import os
import re
import subprocess

import numpy as np
import pytest

import build_ref
import formats_oracle as fo
from oracle import ref_host_lib as orc_ref_host
from conftest import ROOT

# The reference's Code/ folder (GI_REFERENCE_DIR, see oracle/build_ref.py);
# the tests that read its sources skip where it is absent.
REF = os.path.join(build_ref.reference_dir() or "/nonexistent", "Code")

# Setup files in the reference's layout (a comment line without '=', then
# "Name = value;"), written for these tests.
SETUP_GENERATING = """Spin axis of each body and its rate in revolutions per hour:

InitialSpin1.x = 0.0;
InitialSpin1.y = 0.6;
InitialSpin1.z = 0.8;
InitialSpin1.w = 0.25;

InitialSpin2.x = 1.0;
InitialSpin2.y = 0.0;
InitialSpin2.z = 0.0;
InitialSpin2.w = 0.5;

Body masses as fractions of the Earth mass:
FractionEarthMassOfBody1 = 0.62;
FractionEarthMassOfBody2 = 0.41;

Iron and silicate fractions by mass:
FractionFeBody1 = 0.3;
FractionSiBody1 = 0.7;
FractionFeBody2 = 0.25;
FractionSiBody2 = 0.75;

Damping of each body while it settles:
DampRateBody1 = 6.5;
DampRateBody2 = 7.0;

Elements in the whole run:
TotalNumberOfElements = 1500;

Settling phases in hours:
DampTime = 2.0;
DampRestTime = 1.0;
SpinRestTime = 1.5;

Time step in code units:
Dt = 0.004;

Densities in kg per cubic km:
DensityFe = 7.9e12;
DensitySi = 3.3e12;

Push-back strengths:
KFe = 1.2e14;
KSi = 1.4e14;

Push-back reductions:
KRFe = 0.02;
KRSi = 0.015;

Shell depths:
SDFe = 0.01;
SDSi = 0.003;

Screen refresh:
DrawRate = 25;
"""

SETUP_IMPACT_INIT = """Offsets of the bodies in km:
InitialPosition1.x = -30000.0;
InitialPosition1.y = 150.5;
InitialPosition1.z = -900.0;
InitialPosition2.x = 31000.0;
InitialPosition2.y = -150.5;
InitialPosition2.z = 905.25;
Velocities in km/s:
InitialVelocity1.x = 6.5;
InitialVelocity1.y = 0.1;
InitialVelocity1.z = 0.0;
InitialVelocity2.x = -6.75;
InitialVelocity2.y = 0.0;
InitialVelocity2.z = -0.2;
"""

SETUP_ADD_TIME = """* days to add
AdditionTime = 0.25;
* step
Dt = 0.003;
* screen refresh
DrawRate = 10;
* frames
RecordRate = 7;
* recentre
RecenterRate = 11;
"""


def write(tmp_path, name, text):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def setup_dict(s) -> dict:
    d = {f: getattr(s, f) for f, _ in s._fields_}
    d["spin1"], d["spin2"] = list(s.spin1), list(s.spin2)
    return d


def body_dict(b) -> dict:
    return {f: getattr(b, f) for f, _ in b._fields_}


# --------------------------------------------------------------- layouts --

STRUCTS = {
    "gi_setup_generating": "SetupGenerating", "gi_setup_impact_init": "SetupImpactInit",
    "gi_setup_add_time": "SetupAddTime", "gi_body_params": "BodyParams",
    "gi_generation_plan": "GenerationPlan", "gi_earth_moon": "EarthMoon",
    "gi_generate_report": "GenerateReport", "gi_add_time_report": "AddTimeReport",
    "gi_disk_info": "DiskInfo", "gi_options": "Options", "gi_view": "View",
    "gi_server_config": "ServerConfig",
}


def test_struct_layouts_match_header(gi, tmp_path):
    """ctypes mirrors of the new structs have the C compiler's sizes and offsets."""
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "gi_api.h"', "int main(void){"]
    for cname, pyname in STRUCTS.items():
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for f, _ in getattr(gi, pyname)._fields_:
            lines.append(f'printf("{cname}.{f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0;}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = dict(line.rsplit(" ", 1) for line in out if line)
    for cname, pyname in STRUCTS.items():
        cls = getattr(gi, pyname)
        assert int(got[cname]) == C.sizeof(cls), cname
        for f, _ in cls._fields_:
            assert int(got[f"{cname}.{f}"]) == getattr(cls, f).offset, (cname, f)


# --------------------------------------------------------- setup readers --

def test_read_setup_generating_matches_ordered_parse(gi, tmp_path):
    path = write(tmp_path, "setupGeneratingTargetImpactor", SETUP_GENERATING)
    s = setup_dict(gi.read_setup_generating(path))
    vals = fo.ordered_values(SETUP_GENERATING, fo.GENERATING_KINDS)
    mine = (s["spin1"] + s["spin2"] + [s[k] for k in (
        "frac_earth_mass1", "frac_earth_mass2", "frac_fe1", "frac_si1", "frac_fe2", "frac_si2",
        "damp1", "damp2", "n", "damp_time", "damp_rest_time", "spin_rest_time", "dt", "density_fe",
        "density_si", "k_fe", "k_si", "kr_fe", "kr_si", "sd_fe", "sd_si", "draw_rate")])
    assert mine == vals
    assert s["n"] == 1500 and s["draw_rate"] == 25
    assert s["spin1"][1] == np.float32(0.6)  # parsed as float, not double rounded to float


def test_readers_ignore_key_names_and_report_errors(gi, tmp_path):
    renamed = re.sub(r"\b[A-Za-z0-9.]+ =", "whatever =", SETUP_IMPACT_INIT)
    a = gi.read_setup_impact_init(write(tmp_path, "a", SETUP_IMPACT_INIT))
    b = gi.read_setup_impact_init(write(tmp_path, "b", renamed))
    assert list(a.pos2) == list(b.pos2) and list(a.vel2) == list(b.vel2)
    assert list(a.pos2) == [np.float32(31000.0), np.float32(-150.5), np.float32(905.25)]
    t = gi.read_setup_add_time(write(tmp_path, "c", SETUP_ADD_TIME))
    assert (t.additional_time_days, t.dt, t.draw_rate, t.record_rate, t.recenter_rate) == (
        0.25, 0.003, 10, 7, 11)
    with pytest.raises(gi.GIError) as e:  # truncated: the fifth value is missing
        gi.read_setup_add_time(write(tmp_path, "d", SETUP_ADD_TIME.split("RecenterRate")[0]))
    assert e.value.status == 10
    with pytest.raises(gi.GIError) as e:  # not a number
        gi.read_setup_add_time(write(tmp_path, "e", SETUP_ADD_TIME.replace("0.003", "fast")))
    assert e.value.status == 10
    with pytest.raises(gi.GIError) as e:
        gi.read_setup_add_time(str(tmp_path / "missing"))
    assert e.value.status == 9


@pytest.mark.skipif(not os.path.isdir(REF), reason="reference sources not present")
def test_reference_setup_templates_parse(gi):
    """The reference's own setup templates read with the reference's order."""
    t = f"{REF}/../SetupTemplates"
    s = setup_dict(gi.read_setup_generating(f"{t}/setupGeneratingTargetImpactor"))
    text = open(f"{t}/setupGeneratingTargetImpactor").read()
    vals = fo.ordered_values(text, fo.GENERATING_KINDS)
    assert s["spin1"] + s["spin2"] == vals[:8] and s["n"] == vals[16] and s["draw_rate"] == vals[-1]
    i = gi.read_setup_impact_init(f"{t}/setupImpactInitialization")
    vals = fo.ordered_values(open(f"{t}/setupImpactInitialization").read(), "f" * 12)
    assert list(i.pos1) + list(i.pos2) + list(i.vel1) + list(i.vel2) == vals
    a = gi.read_setup_add_time(f"{t}/setupImpactAddTime")
    vals = fo.ordered_values(open(f"{t}/setupImpactAddTime").read(), "ddiii")
    assert [a.additional_time_days, a.dt, a.draw_rate, a.record_rate, a.recenter_rate] == vals


# ------------------------------------------------------------------ units --

def test_derive_units_matches_restatement(gi, tmp_path):
    setup = gi.read_setup_generating(write(tmp_path, "s", SETUP_GENERATING))
    plan = gi.derive_units(setup)
    want = fo.derive_units(setup_dict(setup))
    b = body_dict(plan.body)
    for k in ("unit_time", "unit_length", "unit_mass", "mass_fe", "mass_si", "k_fe", "k_si", "n",
              "nfe1", "nsi1", "nfe2", "nsi2"):
        assert b[k] == want[k], k
    for k in ("mass_body1", "mass_body2", "damp_time", "damp_rest_time", "spin_rest_time",
              "spin1_w", "spin2_w"):
        assert getattr(plan, k) == want[k], k
    # G = 1 in code units: t^2 G m / l^3 == 1, and D = 1 is the Si element diameter
    g_code = fo.UNIVERSAL_GRAVITY * b["unit_time"] ** 2 * b["unit_mass"] / b["unit_length"] ** 3
    # (to the extent the element counts' truncation lets it)
    assert abs(g_code - 1.0) < 1e-2
    assert b["nfe1"] + b["nsi1"] + b["nfe2"] + b["nsi2"] == 1500


def test_derive_units_rejects_bad_fractions(gi, tmp_path):
    bad = SETUP_GENERATING.replace("FractionSiBody2 = 0.75", "FractionSiBody2 = 0.70")
    with pytest.raises(gi.GIError) as e:
        gi.derive_units(gi.read_setup_generating(write(tmp_path, "s", bad)))
    assert e.value.status == 8


def test_kernel_consts_from_body_params(gi, tmp_path):
    plan = gi.derive_units(gi.read_setup_generating(write(tmp_path, "s", SETUP_GENERATING)))
    b = plan.body
    fc, mc = gi.collision_consts_from_body_params(b, 0.004)
    f = np.float32
    assert fc.GMassFeFe == f(b.mass_fe * b.mass_fe) and fc.GMassFeSi == f(b.mass_fe)
    assert fc.KFeFe == f(2 * b.k_fe) and fc.KFeSi == f(b.k_fe + b.k_si)
    assert fc.KRMix == f(b.k_fe + b.k_si * b.kr_si)  # SDFe >= SDSi
    assert fc.ShellBreakFeSi1 == f(1 - b.sd_si) and fc.ShellBreakFeSi2 == f(1 - b.sd_fe)
    assert fc.NFe == b.nfe1 + b.nfe2 and mc.NFe == fc.NFe
    assert mc.Dt == f(0.004) and mc.DtOverMassFe == f(0.004 / b.mass_fe)
    sc, sm = gi.separate_consts_from_body_params(b, 0.004)
    assert (sc.boarder1, sc.boarder2, sc.boarder3) == (b.nfe1, b.nfe1 + b.nsi1,
                                                      b.nfe1 + b.nsi1 + b.nfe2)
    assert (sm.boarder1, sm.boarder2, sm.boarder3) == (sc.boarder1, sc.boarder2, sc.boarder3)
    assert sc.GMassFeSi == f(b.mass_fe * b.mass_si)
    p = gi.params_from_separate_consts(sc)
    assert p.GMassSiSi == 1.0 and p.KRMix == sc.KRMix


# ---------------------------------------------------------- binary files --

def test_body_file_round_trip_and_layout(gi, tmp_path):
    rng = np.random.default_rng(3)
    pos = rng.normal(size=(77, 4)).astype(np.float32)
    vel = rng.normal(size=(77, 4)).astype(np.float32)
    path = str(tmp_path / "targetImpactorInitialPosVel")
    gi.write_body_file(path, pos, vel)
    raw = open(path, "rb").read()
    assert raw == np.int32(77).tobytes() + pos.tobytes() + vel.tobytes()
    p2, v2 = gi.read_body_file(path)
    assert np.array_equal(p2, pos) and np.array_equal(v2, vel)
    open(path, "wb").write(raw[:-4])
    with pytest.raises(gi.GIError) as e:
        gi.read_body_file(path)
    assert e.value.status == 10


def test_frames_append_count_resume(gi, tmp_path):
    rng = np.random.default_rng(4)
    path = str(tmp_path / "impactPosVel")
    n = 33
    frames = [(np.float32(0.5 * k), rng.normal(size=(n, 4)).astype(np.float32),
               rng.normal(size=(n, 4)).astype(np.float32)) for k in range(4)]
    for t, p, v in frames:
        gi.frames_append(path, float(t), p, v)
    raw = open(path, "rb").read()
    assert raw == b"".join(t.tobytes() + p.tobytes() + v.tobytes() for t, p, v in frames)
    assert gi.frames_count(path, n) == 4
    t, p, v = gi.frames_read(path, n)  # the last frame: where a resumed run starts
    assert t == frames[-1][0] and np.array_equal(p, frames[-1][1]) and np.array_equal(v, frames[-1][2])
    t, p, _ = gi.frames_read(path, n, 1)
    assert t == frames[1][0] and np.array_equal(p, frames[1][1])
    with pytest.raises(gi.GIError):
        gi.frames_read(path, n, 4)
    open(path, "ab").write(b"\0" * 10)  # a partly written frame
    with pytest.raises(gi.GIError) as e:
        gi.frames_count(path, n)
    assert e.value.status == 10


# ----------------------------------------------------------- body builder --

def _plan(gi, tmp_path, text=SETUP_GENERATING):
    setup = gi.read_setup_generating(write(tmp_path, "setup", text))
    return setup, gi.derive_units(setup)


def test_raw_bodies_geometry(gi, tmp_path):
    setup, plan = _plan(gi, tmp_path)
    b = plan.body
    pos, vel, redraws = gi.raw_bodies(11, b)
    pos2, _, _ = gi.raw_bodies(11, b)
    pos3, _, _ = gi.raw_bodies(12, b)
    assert np.array_equal(pos, pos2) and not np.array_equal(pos, pos3)
    assert redraws >= 0
    bd = body_dict(b)
    for body in (1, 2):
        s, m, e = fo.body_ranges(bd, body)
        nfe, nall = m - s, e - s
        r1 = (nfe / 0.68 * 2.0) ** (1 / 3)
        r2 = (nall / 0.68 * 2.0) ** (1 / 3)
        rfe = np.linalg.norm(pos[s:m, :3].astype(np.float64), axis=1)
        rsi = np.linalg.norm(pos[m:e, :3].astype(np.float64), axis=1)
        assert rfe.max() <= r1 * (1 + 1e-6)
        assert rsi.min() >= (r1 + 1.0) * (1 - 1e-6) and rsi.max() <= (r2 + 1.0) * (1 + 1e-6)
        assert np.all(pos[s:m, 3] == 2 * (body - 1)) and np.all(pos[m:e, 3] == 2 * (body - 1) + 1)
        assert np.all(vel[s:e, :3] == 0)
        assert np.allclose(vel[s:m, 3], b.mass_fe) and np.all(vel[m:e, 3] == b.mass_si)
        for lo, hi in ((s, m), (m, e)):  # no two elements of a group closer than D
            q = pos[lo:hi, :3]
            d = q[:, None, :] - q[None, :, :]  # float32, as the reference
            sep = np.sqrt((d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]) + d[..., 2] * d[..., 2])
            np.fill_diagonal(sep, np.float32(9.0))
            assert sep.min() >= 1.0


def test_raw_bodies_same_bytes_on_every_host(gi, tmp_path):
    _, plan = _plan(gi, tmp_path)
    pos, vel, redraws = gi.raw_bodies(5, plan.body)
    h = hashlib.sha256(pos.tobytes() + vel.tobytes()).hexdigest()
    assert h == RAW_BODIES_SHA256, h


RAW_BODIES_SHA256 = "deb926118dde7dc7c04fcd8b0c440de68a395a4fc653b1f0ea54473b4f0e18e3"


def test_spin_and_drift_match_restatement(gi, tmp_path):
    setup, plan = _plan(gi, tmp_path)
    b = body_dict(plan.body)
    totals = (plan.mass_body1, plan.mass_body2)
    pos, vel, _ = gi.raw_bodies(21, plan.body)
    rng = np.random.default_rng(21)
    vel[:, :3] = rng.normal(scale=0.05, size=(len(vel), 3)).astype(np.float32)
    mp, mv = pos.copy(), vel.copy()
    op, ov = pos.copy(), vel.copy()
    for body, axis, w in ((1, list(setup.spin1[:3]), plan.spin1_w),
                          (2, list(setup.spin2[:3]), plan.spin2_w)):
        gi.spin_body(mp, mv, plan, body, axis, w)
        fo.spin_body(op, ov, b, totals[body - 1], body, axis, w)
    assert np.array_equal(mv, ov)
    assert not np.array_equal(mv, vel)
    gi.zero_drift(mp, mv, plan)
    fo.zero_drift(op, ov, b, totals)
    assert np.array_equal(mp, op) and np.array_equal(mv, ov)
    with pytest.raises(gi.GIError) as e:
        gi.spin_body(mp, mv, plan, 1, [0.0, 0.0, 0.0], 1.0)
    assert e.value.status == 8


def test_impact_initial_conditions_and_stats(gi, tmp_path):
    _, plan = _plan(gi, tmp_path)
    b = plan.body
    pos, vel, _ = gi.raw_bodies(31, b)
    rng = np.random.default_rng(31)
    vel[:, :3] = rng.normal(scale=0.02, size=(len(vel), 3)).astype(np.float32)
    s = gi.read_setup_impact_init(write(tmp_path, "i", SETUP_IMPACT_INIT))
    sd = {"pos1": list(s.pos1), "pos2": list(s.pos2), "vel1": list(s.vel1), "vel2": list(s.vel2)}
    P, V = gi.impact_initial_conditions(b, s, pos, vel)
    OP, OV = fo.impact_initial_conditions(body_dict(b), sd, pos, vel)
    assert np.array_equal(P, OP) and np.array_equal(V, OV)
    nfe = b.nfe1 + b.nfe2
    # material by index after the reorder: tags 0 / 2 (Fe) first, then 1 / 3
    assert set(P[:nfe, 3].tolist()) <= {0.0, 2.0} and set(P[nfe:, 3].tolist()) <= {1.0, 3.0}
    st = gi.system_stats_host(P, V, nfe, b.mass_fe, b.mass_si)
    want = fo.system_stats(P, V, nfe, b.mass_fe, b.mass_si)
    assert st == want


# ------------------------------------ host steps vs the reference's own code --

needs_ref_host = pytest.mark.skipif(
    orc_ref_host() is None, reason="the reference's host steps are not built (no cut available)")


@needs_ref_host
def test_spin_and_drift_bitwise_vs_reference_code(gi, tmp_path):
    """gi_spin_body and gi_zero_drift against the reference's own spinBody and
    zeroOutTargetImpactorDrift (generateTargetImpactorBasicFunctions.h:
    407-506), compiled from its sources, on the same bodies: every bit."""
    import ctypes as C
    ref = orc_ref_host()
    setup, plan = _plan(gi, tmp_path)
    b = plan.body
    counts = (C.c_int * 4)(b.nfe1, b.nsi1, b.nfe2, b.nsi2)
    for seed in (41, 42):
        pos, vel, _ = gi.raw_bodies(seed, b)
        rng = np.random.default_rng(seed)
        vel[:, :3] = rng.normal(scale=0.05, size=(len(vel), 3)).astype(np.float32)
        mp, mv = pos.copy(), vel.copy()
        rp, rv = pos.copy(), vel.copy()
        for body, axis, w in ((1, list(setup.spin1[:3]), plan.spin1_w),
                              (2, list(setup.spin2[:3]), plan.spin2_w),
                              (1, [0.3, -2.0, 0.5], 0.125)):
            gi.spin_body(mp, mv, plan, body, axis, w)
            spin = (C.c_float * 4)(*axis, w)
            ref.giref_host_spin(rp.ctypes.data, rv.ctypes.data, counts, b.mass_fe, b.mass_si,
                                plan.mass_body1, plan.mass_body2, body, spin)
            assert np.array_equal(mv, rv), (seed, body)
        gi.zero_drift(mp, mv, plan)
        ref.giref_host_zero_drift(rp.ctypes.data, rv.ctypes.data, counts, b.mass_fe, b.mass_si,
                                  plan.mass_body1, plan.mass_body2)
        assert np.array_equal(mp, rp) and np.array_equal(mv, rv)


@needs_ref_host
def test_impact_initial_conditions_bitwise_vs_reference_code(gi, tmp_path):
    """gi_impact_initial_conditions against the reference's own
    readImpactSetupParameters + setupInitialConditions
    (impactInitialization.cu:183-391), compiled from its sources and run in
    a folder laid out as its drivers expect: the same initial frame, bit for
    bit (unit conversion in float, offsets added, [Fe1, Fe2, Si1, Si2])."""
    import ctypes as C
    ref = orc_ref_host()
    _, plan = _plan(gi, tmp_path)
    b = plan.body
    pos, vel, _ = gi.raw_bodies(43, b)
    rng = np.random.default_rng(43)
    vel[:, :3] = rng.normal(scale=0.02, size=(len(vel), 3)).astype(np.float32)
    root = tmp_path / "run"
    (root / "TargetImpactorInformation").mkdir(parents=True)
    work = root / "a" / "b"
    work.mkdir(parents=True)
    gi.write_body_file(str(root / "TargetImpactorInformation" / "targetImpactorInitialPosVel"),
                       pos, vel)
    (root / "setupImpactInitialization").write_text(SETUP_IMPACT_INIT)
    s = gi.read_setup_impact_init(str(root / "setupImpactInitialization"))
    P, V = gi.impact_initial_conditions(b, s, pos, vel)
    RP = np.zeros_like(P)
    RV = np.zeros_like(V)
    counts = (C.c_int * 4)(b.nfe1, b.nsi1, b.nfe2, b.nsi2)
    assert ref.giref_host_impact_setup(str(work).encode(), counts, b.unit_length, b.unit_time,
                                       RP.ctypes.data, RV.ctypes.data) == 0
    assert np.array_equal(P, RP) and np.array_equal(V, RV)


# ------------------------------------------------- writers vs the sources --

def ref_format_lines(path: str, func: str) -> list[str]:
    """The fprintf formats of one reference function, concatenated and split
    into lines."""
    src = open(path, encoding="latin-1").read().replace("\r", "")
    start = re.search(rf"void {func}\s*\([^)]*\)\s*\n\{{", src).start()  # the definition
    end = src.index("\n}\n", start)
    body = src[start:end]
    fmts = re.findall(r'fprintf\s*\(\s*\w+\s*,\s*"((?:[^"\\]|\\.)*)"', body)
    text = "".join(bytes(f, "latin-1").decode("unicode_escape") for f in fmts)
    return text.split("\n")


def line_regex(fmt: str) -> re.Pattern:
    num = {"%f": r"-?(\d+\.\d{6}|nan|inf)", "%lf": r"-?(\d+\.\d{6}|nan|inf)",
           "%e": r"-?(\d\.\d{6}e[-+]\d{2,3}|nan|inf)", "%d": r"-?\d+"}
    parts = re.split(r"(%lf|%f|%e|%d)", fmt)
    return re.compile("".join(num.get(p, re.escape(p)) for p in parts) + r"\Z")


def match_in_order(mine: list[str], ref: list[str]) -> list[int]:
    """Indices of ref lines matched by mine, as an ordered subsequence."""
    pats = [line_regex(f) for f in ref]
    hit, j = [], 0
    for line in mine:
        while j < len(pats) and not pats[j].match(line):
            j += 1
        assert j < len(pats), f"line not in the reference's format: {line!r}"
        hit.append(j)
        j += 1
    return hit


needs_ref = pytest.mark.skipif(not os.path.isdir(REF), reason="reference sources not present")


@needs_ref
def test_parameter_and_centering_writers_match_reference_formats(gi, tmp_path):
    _, plan = _plan(gi, tmp_path)
    p = str(tmp_path / "targetImpactorParameters")
    gi.write_body_params(p, plan.body)
    ref = ref_format_lines(f"{REF}/GenerateTargetImpactorCode/generateTargetImpactorBasicFunctions.h",
                           "recordCarryForwardParameters")
    mine = open(p).read().split("\n")
    assert match_in_order(mine, ref) == list(range(len(ref)))
    back = gi.read_body_params(p)
    for f in ("n", "nfe1", "nsi1", "nfe2", "nsi2"):
        assert getattr(back, f) == getattr(plan.body, f)
    assert back.unit_length == float(f"{plan.body.unit_length:f}")
    v = str(tmp_path / "viewCenteringInfo")
    gi.write_view_centering(v, [1.5, -2.25, 3.0, 0.125, 0.0, -7.5])
    ref = ref_format_lines(f"{REF}/ImpactCode/impactBasicFunctions.h", "recordViewCenteringInfo")
    mine = open(v).read().split("\n")
    assert match_in_order(mine, ref) == list(range(len(ref)))
    assert gi.read_view_centering(v) == [1.5, -2.25, 3.0, 0.125, 0.0, -7.5]


@needs_ref
def test_stats_writers_match_reference_formats(gi, tmp_path):
    setup, plan = _plan(gi, tmp_path)
    pos, vel, _ = gi.raw_bodies(41, plan.body)
    t = str(tmp_path / "targetImpactorStats")
    gi.write_target_impactor_stats(t, plan, setup, setup.dt, pos, vel)
    ref = ref_format_lines(f"{REF}/GenerateTargetImpactorCode/generateTargetImpactorBasicFunctions.h",
                           "recordTargetImpactorStats")
    mine = open(t).read().split("\n")
    assert match_in_order(mine, ref) == list(range(len(ref)))
    b = plan.body
    st = gi.system_stats_host(pos, vel, b.nfe1 + b.nfe2, b.mass_fe, b.mass_si)
    s = str(tmp_path / "initialStatsFile")
    gi.write_initial_stats(s, b, st)
    ref = ref_format_lines(f"{REF}/ImpactCode/impactInitialization.cu", "recordInitialImpactStat")
    mine = open(s).read().split("\n")
    # the reference function goes on to write viewCenteringInfo, a second file
    assert match_in_order(mine, ref) == list(range(len(mine)))
    assert "InitialCenterOfMassX" in ref[len(mine)]
    # final statistics: every line in the reference's order; the lines left
    # out are the alternatives of its if / else branches
    em = gi.EarthMoon(0, 700, 1200, 150, 9, (300, 200, 400, 300), (10, 0, 140, 0))
    S = [[2000.0, 1, 2, 3, 0.1, 0.2, 0.3, 10, 20, 30] + [0] * 5,
         [1500.0, 1, 2, 3, 0.1, 0.2, 0.3, 10, 20, 30] + [0] * 5,
         [1300.0, 1, 2, 3, 0.1, 0.2, 0.3, 10, 20, 30] + [0] * 5,
         [200.0, 4, 5, 6, 0.4, 0.5, 0.6, 1, 2, 3] + [0] * 5]
    r = str(tmp_path / "runStatsFile")
    gi.write_run_stats(r, b, 1234.5, em, S)
    ref = ref_format_lines(f"{REF}/ImpactCode/impactBasicFunctions.h", "recordFinalImpactStat")
    mine = open(r).read().split("\n")
    hit = match_in_order(mine, ref)
    skipped = [ref[k] for k in range(len(ref)) if k not in hit]
    assert all(("composed of" in x) or ("ratio" in x) or x == "" for x in skipped), skipped
    text = open(r).read()
    assert "The Moon is only composed of elements from body 1" in text
    assert "Earth ratio body1/body2" in text and "The mass ratio Earth/Moon" in text
