"""Generates the golden fixtures in this directory from the reference's own code.

Runs the UNMODIFIED reference modules (``cardiax/solve.py``, ``cardiax/stimulus.py``,
``cardiax/params.py``) from a reference checkout, with JAX replaced by the NumPy stand-in of
``ref_shim.py`` (JAX is not installable here).  Usage::

    python tests/golden/make_golden.py [--reference /path/to/cardiax-checkout]

Fixtures (all float32 unless noted; "x64" = the same code with float64, JAX's x64 mode):

* ``stimulus_schedule.json`` -- steps at which the stimuli of the reference's
  ``tests/macro/stimulate_test.py:8-18`` are active, computed with the current
  ``cardiax.solve.stimulate``
* ``params.json``          -- every PARAMSET_* of ``cardiax/params.py``
* ``gradient.npz``         -- ``solve.gradient`` along both axes on small arrays
* ``step.npz``             -- ``solve.step`` derivatives on small grids with stimuli
* ``forward_small.npz``    -- ``solve._forward_euler`` 0 -> 200 on 32x40 (float32 and x64)
* ``heun_small.npz``       -- ``solve._forward_heun`` on the same case (float32 and x64)
* ``config0.npz``          -- ``solve.forward`` on the 128x128 plain configuration (planar
  stimulus on the left 5 columns, amplitude 1.0, Protocol(0, 200, 1e9), checkpoints every
  100 steps to 1000) and its excitable variant (amplitude 20, Protocol(0, 2, 1e9))
* ``paramsets.npz``        -- ``solve.forward`` for 1000 steps (checkpoints every 250: float32
  u at each, v, w, u of both precisions at the last) on a 48x60 grid with a smooth D map, a
  planar (8 columns) and a point (8x8) stimulus, under parameter sets 1A, 4A and 5 (the batched workload's sets besides
  3) and 2 (a set with MAXFLOAT entries), float32 and x64

* ``config0_x64.npz``      -- the configuration-0 runs of ``config0.npz`` with x64 (float64): u
  at 1000 steps, the error reference of the benchmark's parity figures

``--only NAME`` regenerates one fixture group (e.g. ``--only paramsets``) and leaves the other
files untouched.
"""
from __future__ import annotations

import argparse
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

from ref_shim import REFERENCE_ROOT, load_reference  # noqa: E402

SEED = 20261203


def smooth_field(rng, shape, lo, hi, dtype=np.float32):
    """Sum of a few random Gaussian bumps rescaled to [lo, hi] (a smooth map)."""
    H, W = shape
    i, j = np.meshgrid(np.arange(H), np.arange(W), indexing="ij")
    f = np.zeros(shape)
    for _ in range(4):
        ci, cj = rng.uniform(0, H), rng.uniform(0, W)
        s = rng.uniform(0.15, 0.4) * max(H, W)
        f += rng.uniform(-1, 1) * np.exp(-((i - ci) ** 2 + (j - cj) ** 2) / (2 * s * s))
    f = (f - f.min()) / (f.max() - f.min() + 1e-12)
    return (lo + (hi - lo) * f).astype(dtype)


PARAMSET_CASES = ("1A", "4A", "5", "2")


def paramset_fixtures(R, R64, out):
    """``forward`` under parameter sets other than 3 (1000 steps, float32 and x64)."""
    rng = np.random.default_rng(SEED + 1)
    shp = (48, 60)
    D = smooth_field(rng, shp, 3e-4, 1e-3)
    # 8 columns: a narrower 2-step pulse does not start a wave under sets 1A, 4A, 5
    f1 = np.zeros(shp, np.float32)
    f1[:, :8] = 20.0
    f2 = np.zeros(shp, np.float32)
    f2[30:38, 40:48] = 20.0
    ck = np.arange(0, 1001, 250)
    ps = {"D": D, "f1": f1, "f2": f2, "checkpoints": ck}
    for name in PARAMSET_CASES:
        for R_, dt_ in ((R, np.float32), (R64, np.float64)):
            P_ = getattr(R_.params, f"PARAMSET_{name}")
            stims = [R_.stimulus.Stimulus(R_.stimulus.Protocol(0, 2, 1e9), f1.astype(dt_)),
                     R_.stimulus.Stimulus(R_.stimulus.Protocol(300, 2, 1e9), f2.astype(dt_))]
            states = R_.solve.forward(R_.solve.init(shp), ck, P_, D.astype(dt_), stims, 0.01,
                                      0.01)
            print()
            tag = "f32" if dt_ == np.float32 else "f64"
            # float32: u at every checkpoint; both: v, w, u at the last
            for i, st in enumerate(states if tag == "f32" else states[-1:]):
                ps[f"{name}_{tag}_u_{ck[i + 1] if tag == 'f32' else ck[-1]}"] = np.asarray(st.u)
            ps[f"{name}_{tag}_v_{ck[-1]}"] = np.asarray(states[-1].v)
            ps[f"{name}_{tag}_w_{ck[-1]}"] = np.asarray(states[-1].w)
    np.savez_compressed(os.path.join(out, "paramsets.npz"), **ps)


def config0_x64_fixtures(R64, out):
    """The 128x128 configuration (plain and excitable) in float64, u at 1000 steps."""
    shp = (128, 128)
    D = np.full(shp, 0.001, np.float64)
    ck = np.arange(0, 1001, 100)
    c0 = {}
    for tag, amp, proto in (("plain", 1.0, (0, 200, 1e9)), ("excite", 20.0, (0, 2, 1e9))):
        stim = R64.stimulus.linear(shp, R64.stimulus.Direction.WEST, 5 / 128, amp,
                                   R64.stimulus.Protocol(*proto))
        states = R64.solve.forward(R64.solve.init(shp), ck, R64.params.PARAMSET_3, D, [stim],
                                   0.01, 0.01)
        print()
        c0[f"{tag}_u_1000"] = np.asarray(states[-1].u, np.float64)
    np.savez_compressed(os.path.join(out, "config0_x64.npz"), **c0)


def main(root: str, only: str = None):
    R = load_reference(root=root)
    R64 = load_reference(x64=True, root=root)
    S, P = R.solve, R.params
    rng = np.random.default_rng(SEED)
    out = HERE
    if only in ("paramsets", "config0_x64"):
        (paramset_fixtures(R, R64, out) if only == "paramsets" else config0_x64_fixtures(R64, out))
        print("fixtures written to", out)
        return
    if only is not None:
        raise SystemExit(f"unknown fixture group {only!r}")

    # --- stimulus schedule (tests/macro/stimulate_test.py:8-18, current stimulate) ---------
    shape = (16, 16)
    field = np.ones(shape, np.float32)
    protos = {"A": (0, 2, 50), "B": (10, 2, 50), "C": (30, 2, 1000000)}
    sched = {}
    for name, pr in protos.items():
        st = [R.stimulus.Stimulus(R.stimulus.Protocol(*pr), field)]
        on = []
        for t in range(300):
            X = S.stimulate(np.float32(t), np.zeros(shape, np.float32), st)
            if np.any(X != 0):
                on.append(t)
        sched[name] = {"protocol": pr, "active": on}
    extra = {"quirk_long_duration": (0, 200, 1e9), "quirk_periodic": (10, 5, 20)}
    for name, pr in extra.items():
        st = [R.stimulus.Stimulus(R.stimulus.Protocol(*pr), field)]
        sched[name] = {"protocol": pr, "active": [t for t in range(300) if np.any(
            S.stimulate(np.float32(t), np.zeros(shape, np.float32), st) != 0)]}
    with open(os.path.join(out, "stimulus_schedule.json"), "w") as f:
        json.dump(sched, f, indent=1)

    # --- parameter sets ----------------------------------------------------------------------
    sets = {k: list(map(float, getattr(P, k))) for k in dir(P) if k.startswith("PARAMSET_")}
    with open(os.path.join(out, "params.json"), "w") as f:
        json.dump({"fields": list(P.Params._fields), "sets": sets}, f, indent=1)

    # --- gradient ------------------------------------------------------------------------------
    g = {}
    for k, shp in enumerate([(5, 5), (5, 8), (9, 7), (12, 17)]):
        a = rng.standard_normal(shp).astype(np.float32)
        g[f"in{k}"] = a
        g[f"ax0_{k}"] = S.gradient(a, 0)
        g[f"ax1_{k}"] = S.gradient(a, 1)
    np.savez_compressed(os.path.join(out, "gradient.npz"), **g)

    # --- step (derivative) --------------------------------------------------------------------
    st_cases = {}
    for k, shp in enumerate([(3, 3), (5, 9), (17, 23), (32, 32)]):
        v = smooth_field(rng, shp, 0.0, 1.0)
        w = smooth_field(rng, shp, 0.0, 1.0)
        u = smooth_field(rng, shp, 0.0, 1.0)
        D = smooth_field(rng, shp, 2e-4, 1e-3)
        f1 = np.zeros(shp, np.float32)
        f1[:, : max(1, shp[1] // 5)] = 20.0
        f2 = np.zeros(shp, np.float32)
        f2[shp[0] // 3: shp[0] // 3 + 2, 1:3] = 5.0
        stims = [R.stimulus.Stimulus(R.stimulus.Protocol(0, 2, 1e9), f1),
                 R.stimulus.Stimulus(R.stimulus.Protocol(1, 3, 7), f2)]
        for t in (0, 1, 5):
            d = S.step(S.State(v, w, u), np.float32(t), P.PARAMSET_3, D, stims, 0.01)
            for name, arr in zip(("dv", "dw", "du"), d):
                st_cases[f"{name}_{k}_{t}"] = arr
        st_cases.update({f"v_{k}": v, f"w_{k}": w, f"u_{k}": u, f"D_{k}": D,
                         f"f1_{k}": f1, f"f2_{k}": f2})
    np.savez_compressed(os.path.join(out, "step.npz"), **st_cases)

    # --- forward_euler on a small grid, float32 and x64 ---------------------------------------
    shp = (32, 40)
    D = smooth_field(rng, shp, 3e-4, 1e-3)
    f1 = np.zeros(shp, np.float32)
    f1[:, :4] = 20.0
    f2 = np.zeros(shp, np.float32)
    f2[20:26, 30:36] = 10.0
    fs = {}
    for R_, dt_ in ((R, np.float32), (R64, np.float64)):
        stims = [R_.stimulus.Stimulus(R_.stimulus.Protocol(0, 2, 1e9), f1.astype(dt_)),
                 R_.stimulus.Stimulus(R_.stimulus.Protocol(60, 3, 1e9), f2.astype(dt_))]
        st = R_.solve.init(shp)
        res = R_.solve._forward_euler(st, 0.0, 200.0, P.PARAMSET_3, D.astype(dt_), stims, 0.01,
                                      0.01)
        tag = "f32" if dt_ == np.float32 else "f64"
        for name, arr in zip("vwu", res):
            fs[f"{name}_{tag}"] = arr
    fs.update({"D": D, "f1": f1, "f2": f2})
    np.savez_compressed(os.path.join(out, "forward_small.npz"), **fs)

    # --- Heun integrator on the same small case (cardiax/solve.py:73-85,103-111) -------------
    hs = {}
    for R_, dt_ in ((R, np.float32), (R64, np.float64)):
        stims = [R_.stimulus.Stimulus(R_.stimulus.Protocol(0, 2, 1e9), f1.astype(dt_)),
                 R_.stimulus.Stimulus(R_.stimulus.Protocol(60, 3, 1e9), f2.astype(dt_))]
        res = R_.solve._forward_heun(R_.solve.init(shp), 0.0, 200.0, P.PARAMSET_3,
                                     D.astype(dt_), stims, 0.01, 0.01)
        tag = "f32" if dt_ == np.float32 else "f64"
        for name, arr in zip("vwu", res):
            hs[f"{name}_{tag}"] = arr
    np.savez_compressed(os.path.join(out, "heun_small.npz"), **hs)

    # --- configuration 0 (128x128, 1000 steps) and its excitable variant ---------------------
    shp = (128, 128)
    D = np.full(shp, 0.001, np.float32)
    ck = np.arange(0, 1001, 100)
    c0 = {}
    for tag, amp, proto in (("plain", 1.0, (0, 200, 1e9)), ("excite", 20.0, (0, 2, 1e9))):
        stim = R.stimulus.linear(shp, R.stimulus.Direction.WEST, 5 / 128, amp,
                                 R.stimulus.Protocol(*proto))
        states = S.forward(S.init(shp), ck, P.PARAMSET_3, D, [stim], 0.01, 0.01)
        print()
        for i, s in enumerate(states):
            c0[f"{tag}_u_{ck[i + 1]}"] = s.u
        c0[f"{tag}_v_final"], c0[f"{tag}_w_final"] = states[-1].v, states[-1].w
        c0[f"{tag}_field"] = np.asarray(stim.field)
    np.savez_compressed(os.path.join(out, "config0.npz"), **c0)
    config0_x64_fixtures(R64, out)
    paramset_fixtures(R, R64, out)
    print("fixtures written to", out)


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=REFERENCE_ROOT, required=REFERENCE_ROOT is None,
                    help="reference checkout (default: $CARDIAX_REFERENCE)")
    ap.add_argument("--only", default=None,
                    help="regenerate one fixture group (paramsets, config0_x64)")
    a = ap.parse_args()
    main(a.reference, a.only)
