"""CPU restatement of the Giant-Impact host steps around the force path:
setup-file parsing, unit derivation, spin, drift removal, impact initial
conditions and the initial statistics.

TEST INFRASTRUCTURE, NOT PRODUCT CODE.  Only tests/ import this module.  It
follows the reference's host code statement by statement in numpy with the
reference's types (float32 positions and velocities, float64 sums in index
order), so that the library's C++ versions can be compared bit for bit.
"""
from __future__ import annotations

import math
import re

import numpy as np

PI = 3.141592654            # commonSetup.h:29
UNIVERSAL_GRAVITY = 6.67408e-20  # commonSetup.h:31
MASS_OF_EARTH = 5.97219e24  # commonSetup.h:33
RADIUS_OF_EARTH = 6378.0    # commonSetup.h:35

f32 = np.float32


def ordered_values(text: str, kinds: str) -> list:
    """getline(data, name, '=') then data >> value, once per character of
    kinds ('f' float, 'd' double, 'i' int) -- generateTargetImpactor.cu:169-248.
    Raises ValueError where the stream would fail."""
    out = []
    at = 0
    num = {"f": r"[-+]?(\d+\.?\d*|\.\d+)([eE][-+]?\d+)?", "d": None, "i": r"[-+]?\d+"}
    num["d"] = num["f"]
    for k in kinds:
        eq = text.find("=", at)
        if eq < 0:
            raise ValueError("missing '='")
        at = eq + 1
        while at < len(text) and text[at].isspace():
            at += 1
        m = re.match(num[k], text[at:])
        if not m:
            raise ValueError("not a number")
        at += m.end()
        tok = m.group(0)
        out.append(int(tok) if k == "i" else (float(f32(float(tok))) if k == "f" else float(tok)))
    return out


GENERATING_KINDS = "ffff" "ffff" "dd" "dddd" "ff" "i" "ddd" "d" "dd" "dd" "dd" "dd" "i"


def derive_units(s: dict) -> dict:
    """setTargetImpactorParameters (generateTargetImpactor.cu:289-403)."""
    mb1 = MASS_OF_EARTH * s["frac_earth_mass1"]
    mb2 = MASS_OF_EARTH * s["frac_earth_mass2"]
    fe1, si1 = s["frac_fe1"] * mb1, s["frac_si1"] * mb1
    fe2, si2 = s["frac_fe2"] * mb2, s["frac_si2"] * mb2
    fe, si = fe1 + fe2, si1 + si2
    rho = s["density_si"] / s["density_fe"]
    nfe = int(float(s["n"]) * rho / (si / fe + rho)) if fe != 0.0 else 0
    nsi = s["n"] - nfe
    nfe1 = int(nfe * fe1 / fe) if fe != 0.0 else 0
    nsi1 = int(nsi * si1 / si) if si != 0.0 else 0
    msi = si / nsi
    ul = math.pow((6.0 * msi) / (PI * s["density_si"]), 1.0 / 3.0)
    um = msi
    ut = math.sqrt((6.0 * msi * float(nsi)) / (UNIVERSAL_GRAVITY * PI * s["density_si"] * si))
    return dict(unit_time=ut, unit_length=ul, unit_mass=um, diameter=1.0, mass_si=1.0,
                mass_fe=s["density_fe"] / s["density_si"],
                k_fe=s["k_fe"] * ut * ut * ul / um, k_si=s["k_si"] * ut * ut * ul / um,
                n=s["n"], nfe1=nfe1, nsi1=nsi1, nfe2=nfe - nfe1, nsi2=nsi - nsi1,
                mass_body1=mb1 / um, mass_body2=mb2 / um,
                damp_time=s["damp_time"] * 3600.0 / ut,
                damp_rest_time=s["damp_rest_time"] * 3600.0 / ut,
                spin_rest_time=s["spin_rest_time"] * 3600.0 / ut,
                spin1_w=float(f32(float(s["spin1"][3]) * (ut / 3600.0))),
                spin2_w=float(f32(float(s["spin2"][3]) * (ut / 3600.0))))


def _seq_sum(terms: np.ndarray) -> float:
    """Sum in index order (np.add.accumulate is sequential)."""
    return float(np.add.accumulate(terms)[-1]) if len(terms) else 0.0


def body_ranges(b: dict, body: int):
    if body == 1:
        return 0, b["nfe1"], b["nfe1"] + b["nsi1"]
    o = b["nfe1"] + b["nsi1"]
    return o, o + b["nfe2"], o + b["nfe2"] + b["nsi2"]


def body_mean(a: np.ndarray, b: dict, total: float, body: int) -> list[float]:
    """getCenterOfMass / getAverageLinearVelocity
    (generateTargetImpactorBasicFunctions.h:29-80, :119-171)."""
    if total < 0.00000000001:
        return [0.0, 0.0, 0.0]
    s, m, e = body_ranges(b, body)
    out = []
    for c in range(3):
        terms = np.concatenate([a[s:m, c].astype(np.float64) * b["mass_fe"],
                                a[m:e, c].astype(np.float64) * b["mass_si"]])
        out.append(_seq_sum(terms) / total)
    return out


def spin_body(pos, vel, b: dict, total: float, body: int, axis, w: float) -> None:
    """spinBody (generateTargetImpactorBasicFunctions.h:407-470), in place."""
    ax = np.array(axis, dtype=np.float32)
    mag = float(np.sqrt(f32(f32(ax[0] * ax[0]) + f32(ax[1] * ax[1])) + f32(ax[2] * ax[2])))
    s = [float(f32(float(x) / mag)) for x in ax]
    com = body_mean(pos, b, total, body)
    st, _, e = body_ranges(b, body)
    for i in range(st, e):
        rx, ry, rz = (float(pos[i, k]) - com[k] for k in range(3))
        mag2 = rx * rx + ry * ry + rz * rz
        along = s[0] * rx + s[1] * ry + s[2] * rz
        perp2 = mag2 - along * along
        perp = math.sqrt(perp2) if perp2 > 0.0 else 0.0
        speed = float(f32(w)) * 2.0 * PI * perp
        nx = s[1] * rz - s[2] * ry
        ny = -(s[0] * rz - s[2] * rx)
        nz = s[0] * ry - s[1] * rx
        nm = math.sqrt(nx * nx + ny * ny + nz * nz)
        if nm != 0.0:
            nx, ny, nz = nx / nm, ny / nm, nz / nm
            vel[i, 0] = f32(float(vel[i, 0]) + speed * nx)
            vel[i, 1] = f32(float(vel[i, 1]) + speed * ny)
            vel[i, 2] = f32(float(vel[i, 2]) + speed * nz)


def zero_drift(pos, vel, b: dict, totals) -> None:
    """zeroOutTargetImpactorDrift (generateTargetImpactorBasicFunctions.h:472-506)."""
    for body in (1, 2):
        c = body_mean(pos, b, totals[body - 1], body)
        u = body_mean(vel, b, totals[body - 1], body)
        s, _, e = body_ranges(b, body)
        for k in range(3):
            pos[s:e, k] = (pos[s:e, k].astype(np.float64) - c[k]).astype(np.float32)
            vel[s:e, k] = (vel[s:e, k].astype(np.float64) - u[k]).astype(np.float32)


def impact_initial_conditions(b: dict, setup: dict, pos, vel):
    """setupInitialConditions (impactInitialization.cu:260-371)."""
    n1 = b["nfe1"] + b["nsi1"]
    tp, tv = pos.copy(), vel.copy()
    for body, sl in ((0, slice(0, n1)), (1, slice(n1, b["n"]))):
        for k in range(3):
            dp = f32(float(f32(setup[f"pos{body + 1}"][k])) / b["unit_length"])
            dv = f32(float(f32(setup[f"vel{body + 1}"][k])) * (b["unit_time"] / b["unit_length"]))
            tp[sl, k] = tp[sl, k] + dp
            tv[sl, k] = tv[sl, k] + dv
    nfe1, nfe2 = b["nfe1"], b["nfe2"]
    order = np.concatenate([np.arange(0, nfe1), np.arange(n1, n1 + nfe2), np.arange(nfe1, n1),
                            np.arange(n1 + nfe2, b["n"])])
    return tp[order], tv[order]


def system_stats(pos, vel, nfe: int, mass_fe: float, mass_si: float) -> list[float]:
    """recordInitialImpactStat (impactInitialization.cu:393-474)."""
    n = len(pos)
    m = np.where(np.arange(n) < nfe, mass_fe, mass_si).astype(np.float64)
    M = _seq_sum(m)
    c = [_seq_sum(pos[:, k].astype(np.float64) * m) / M for k in range(3)]
    u = [_seq_sum(vel[:, k].astype(np.float64) * m) / M for k in range(3)]
    r = pos[:, :3].astype(np.float64) - np.array(c)
    v = vel[:, :3].astype(np.float64) - np.array(u)
    L = [_seq_sum((r[:, 1] * v[:, 2] - r[:, 2] * v[:, 1]) * m),
         _seq_sum(-(r[:, 0] * v[:, 2] - r[:, 2] * v[:, 0]) * m),
         _seq_sum((r[:, 0] * v[:, 1] - r[:, 1] * v[:, 0]) * m)]
    return [M] + c + u + L


def generate_phase_counts(dt: float, damp_time: float, damp_rest_time: float,
                          spin_rest_time: float) -> list[int]:
    """Steps of the damped, damped-rest and spin-rest phases of the body
    builder: RunTime += Dt, then the phase test, then the end test
    (generateTargetImpactor.cu:666-749)."""
    t, count = 0.0, [0, 0, 0]
    end = damp_time + damp_rest_time + spin_rest_time
    while True:
        t += dt
        count[0 if t < damp_time else (1 if t < damp_time + damp_rest_time else 2)] += 1
        if end < t:
            return count


def add_time_events(t0: float, additional: float, dt: float, record_rate: int,
                    recenter_rate: int) -> list[tuple]:
    """(step, run_time, record, recenter) of every step of an impact run that
    records or recenters, and the last step (impactAddTime.cu:396-481)."""
    t, total, k = t0, t0 + additional, 0
    rc = cc = 0
    out = []
    while True:
        k += 1
        t += dt
        rc += 1
        cc += 1
        rec, cen, done = rc == record_rate, cc == recenter_rate, total < t
        if rec:
            rc = 0
        if cen:
            cc = 0
        if rec or cen or done:
            out.append((k, t, rec, cen))
        if done:
            return out
