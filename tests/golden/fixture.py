"""Load a golden fixture (reference-kernel run) and replay its inputs through
any library that exports the C ABI (the CUDA engine or the CPU oracle)."""
from __future__ import annotations

import os

import numpy as np

from rift_gb300 import synth

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = ("rain", "h0_infil_src", "front", "gridrain_surge", "euler", "noaccel")


class FixtureCase(synth.Case):
    """A Case whose faces come straight from the fixture (no regeneration)."""

    def __init__(self, fx):
        super().__init__(name="fixture", B=fx["B"], cell=float(fx["cell"]), n=fx["n"],
                         K=fx["K"] if "K" in fx else None, h0=fx["h0"] if "h0" in fx else None,
                         psi=float(fx["psi"]), dtheta=float(fx["dtheta"]),
                         courant=float(fx["courant"]), t0=float(fx["t0"]), flags=int(fx["flags"]))
        self._BX = fx["BX"]
        self._BY = fx["BY"]
        self._kappa = float(fx["kappa"])
        self.series = {}
        for w in range(3):
            if f"series{w}_t" in fx:
                self.series[w] = (fx[f"series{w}_t"], fx[f"series{w}_r"])
        self.src_idx = fx["src_idx"] if "src_idx" in fx else None

    def faces(self):
        return self._BX, self._BY

    @property
    def kappa(self):
        return self._kappa


def load(name):
    fx = dict(np.load(os.path.join(HERE, f"{name}.npz")))
    return fx, FixtureCase(fx)


def start(sim, fx):
    """Upload inputs and maps exactly as the reference run saw them."""
    sim.setup()
    for k, which in (("rain", 0), ("drain", 1), ("surge", 2)):
        if f"map_{k}_mode" in fx:
            mode = int(fx[f"map_{k}_mode"])
            t1 = fx[f"map_{k}_t1"] if mode == 2 else None
            sim.set_map(which, fx[f"map_{k}_t0"], t1, float(fx[f"map_{k}_factor"]))
    return sim


def dumps(fx):
    return [int(s) for s in fx["dumps"]]


def ref_state(fx, step):
    p = f"s{step}_"
    return {k[len(p):]: v for k, v in fx.items() if k.startswith(p)}


def interior(a):
    return a[2:-2, 2:-2]
