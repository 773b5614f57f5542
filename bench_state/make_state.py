"""Writes bench_state/impact66k_seed2.npz, the input state of bench.py's
default workload: the plain two-body impact of a 60,000-body target and a
6,000-body impactor (30 % Fe core each), each built as a seeded ball, settled
on the GPU with the damped separate-body step (1,500 damped steps and 150
undamped rest steps, dt = 1e-3), then spun about z at 0.5 of breakup, placed
at 45 degrees and moving at 1.2 x the mutual escape speed, in the reference's
[Fe1, Fe2, Si1, Si2] order.

Both arms of bench.py read this one file, so they time the identical state,
and the reference arm (the reference's force loop on the host cores) needs
no GPU library to build it.  The settle is deterministic on a given GPU
model, so rerunning this script reproduces the file bit for bit there.

  python bench_state/make_state.py [out.npz]     (needs a GPU)
"""
from __future__ import annotations

import importlib.util
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
PKG = os.path.join(ROOT, "giant-impact_gb300")
OUT = os.path.join(HERE, "impact66k_seed2.npz")
SEED, SETTLE_STEPS = 2, 1500


def _load(name, path):
    if name in sys.modules:
        return sys.modules[name]
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def main(out=OUT):
    import numpy as np
    import torch
    gi = _load("gi", os.path.join(PKG, "gi.py"))
    wl = _load("gi_workloads", os.path.join(PKG, "gi_workloads.py"))
    pos, vel, nfe = wl.impact(gi, torch, 60000, 6000, seed=SEED, settle_steps=SETTLE_STEPS)
    np.savez_compressed(out, pos=pos, vel=vel, nfe=np.int64(nfe), seed=np.int64(SEED),
                        settle_steps=np.int64(SETTLE_STEPS))
    print(out, len(pos), nfe)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else OUT)
