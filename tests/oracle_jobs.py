"""Oracle runs for the GPU parity tests, shaped for a process pool.

The oracle is single-threaded; the parity tests on the layered 3D slope
need several of its trials, so they run side by side in worker processes
started with ``spawn`` (never forked from a process that has touched the
GPU).  Test infrastructure only.
"""
from __future__ import annotations

import concurrent.futures as cf
import multiprocessing as mp

import numpy as np

# The layered 3D slope class of the 192k-element benchmark mesh (60x20x30 m,
# 1:2 face, three layers, every element its own lognormally perturbed block),
# cut to 24 x 4 x 6 = 576 elements so that the oracle finishes in seconds.
SLOPE3D_CUT = dict(nx=24, ny=4, nz=6)


def slope3d_cut():
    from specfem3d_geotech_gb300 import meshgen
    return meshgen.slope3d(**SLOPE3D_CUT)


def _trial(srf: float):
    from oracle.pyoracle import OracleModel
    om = OracleModel(slope3d_cut())
    r = om.trial(srf, want_x=True, want_stress=True, want_log=True)
    return {k: (np.asarray(v) if isinstance(v, np.ndarray) else v) for k, v in r.items()}


def slope3d_cut_trials(srfs):
    """Oracle trials of the 3D cut at each SRF, run in parallel; {srf: result}."""
    ctx = mp.get_context("spawn")
    with cf.ProcessPoolExecutor(max_workers=len(srfs), mp_context=ctx) as ex:
        return dict(zip(srfs, ex.map(_trial, srfs)))
