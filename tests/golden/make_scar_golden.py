"""Generates ``scars.npz`` from the reference's own ``deepx/utils_scars.py``.

Runs the UNMODIFIED ``random_diffusivity_scar`` (utils_scars.py:409-426) under the stand-ins of
``scar_shim.py`` with scripted random draws, and records per case the draws, the union mask that
reaches ``blur_scar`` and the returned field.  Usage::

    python tests/golden/make_scar_golden.py [--reference /path/to/cardiax-checkout]

Cases: square 64, 100, 128 and 256 grids, the non-square 96x128 and 128x96 (the reference
scales the field with shape[0] / shape[1] and sizes the blur from shape[0]), and a 128 grid
with a blur narrow enough that the Gaussian's far entries fall below eps * max and are zeroed.
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

from scar_shim import REFERENCE_ROOT, Tape, load_utils_scars  # noqa: E402

SEED = 20261204
CASES = [(64, 64), (100, 100), (128, 128), (96, 128), (128, 96), (256, 256), (128, 128)]
# a case whose blur is narrow enough that makegauss2D zeroes the kernel's far entries
NARROW_CASE, NARROW_SIGMA_NORMAL = 6, np.float32(0.04)


def scripted_draws(rng, sigma_normal=None):
    """Draws in the reference's call order (utils_scars.py:224-243, 246-352, 420-424)."""
    c = rng.standard_normal(12).astype(np.float32)
    n = int(rng.integers(3, 7))
    first = int(rng.integers(0, 12))
    blobs = rng.standard_normal((n, 11)).astype(np.float32)
    ux, uy = np.float32(rng.random()), np.float32(rng.random())
    s = np.float32(rng.standard_normal())
    if sigma_normal is not None:
        s = np.float32(sigma_normal)
    tape = [("normal", (12,), c), ("randint", (1,), [n]), ("randint", (1,), [first])]
    tape += [("normal", (11,), b) for b in blobs]
    tape += [("uniform", (), ux), ("uniform", (), uy), ("normal", (1,), [s])]
    return dict(centroid_normals=c, n_blobs=n, first=first, blob_normals=blobs, ux=ux, uy=uy,
                sigma_normal=s), tape


def main(root: str):
    rng = np.random.default_rng(SEED)
    out = {}
    for k, shape in enumerate(CASES):
        draws, items = scripted_draws(rng, NARROW_SIGMA_NORMAL if k == NARROW_CASE else None)
        tape = Tape(items)
        U = load_utils_scars(tape, root)
        seen = {}
        blur = U.blur_scar

        def recording_blur(scar, size, sigma, _blur=blur):
            seen["mask"] = np.array(scar)
            seen["size"], seen["sigma"] = size, np.array(sigma)
            return _blur(scar, size, sigma)

        U.blur_scar = recording_blur
        field = np.asarray(U.random_diffusivity_scar(("key", k), shape), np.float32)
        assert tape.pos == len(tape.items), "unused draws"
        mask = seen["mask"]
        assert set(np.unique(mask)) == {0.0, 1.0}, "degenerate or non-binary mask"
        p = f"c{k}_"
        out[p + "shape"] = np.array(shape)
        for name, v in draws.items():
            out[p + name] = np.asarray(v)
        out[p + "mask"] = np.packbits(mask.astype(np.uint8))
        out[p + "ksize"] = np.array(seen["size"])
        out[p + "sigma"] = seen["sigma"].astype(np.float32)
        out[p + "field"] = field
        print(shape, "blobs", draws["n_blobs"], "cells", int(mask.sum()), "K", seen["size"],
              "sigma", float(seen["sigma"][0]))
    out["n_cases"] = np.array(len(CASES))
    np.savez_compressed(os.path.join(HERE, "scars.npz"), **out)


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=REFERENCE_ROOT, required=REFERENCE_ROOT is None,
                    help="reference checkout (default: $CARDIAX_REFERENCE)")
    main(ap.parse_args().reference)
